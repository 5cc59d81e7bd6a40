// Kernel launchers of the Spiral answer path (host side declarations).
// Every launcher enqueues on `st` and returns the launch status.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#include <utility>

#include "common.cuh"

namespace sp {

// Launch with programmatic stream serialisation when `pdl` (the kernel then
// calls pdl_wait() before touching its predecessor's data), else normally.
template <typename... KArgs, typename... Args>
cudaError_t launch_ex(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                      Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Device layout of one database image: one 28-bit residue per (prime,
// combo, row, slot), where combo m = t*cols + col enumerates the n*n
// plaintext polynomials of every column:
//   [prime][z][combo block][row][combo in block]
// A block holds cb = min(128, combos) combos.  Each (prime, z, block) triple
// ("unit") is one contiguous stream of `rows` packed rows: the first-dimension
// multiply for one slot and prime is the matrix product of that rows x cb
// block with the query selectors of the slot, so a unit is also exactly the
// operand tile of the tensor-core multiply (128 combos x rows).
//
// Both primes are below 2^28, so a row packs every 8 consecutive combos'
// residues into 7 words (bits 28j .. 28j+27 of the group's 224-bit
// little-endian string hold combo 8k+j): 7/8 of the bytes of u32 residues,
// which is what the HBM-bound one-query multiply reads per query.  A row has
// cbp = cb rounded up to 8 combo places (the tail of a row narrower than 8
// combos is zero).
struct DbLayout {
    int T;        // n*n
    int nu1, nu2;
    int rows, cols;
    int combos;   // T*cols
    int cb;       // combos per block
    int ncb;      // combos / cb
    int cbp;      // combo places per packed row (cb rounded up to 8)
    int rw;       // u32 words per packed row (cbp * 7 / 8)
    uint64_t words;  // residue pairs (u64 words of the NTT-form planes) = rows*combos*D
    __host__ __device__ uint64_t units() const { return 2ull * D * ncb; }
    __host__ __device__ uint64_t unit_words32() const { return (uint64_t)rows * rw; }
    __host__ __device__ uint64_t image_bytes() const { return units() * unit_words32() * 4; }
    // first word of (prime, z, block, row)
    __host__ __device__ uint64_t row_offset32(int prime, int z, int block, int row) const {
        return ((((uint64_t)prime * D + z) * ncb + block) * rows + row) * rw;
    }
};

constexpr uint32_t RES_MASK = 0x0fffffffu;   // one 28-bit residue

// The 8 residues of one packed group (7 words).
__device__ __forceinline__ void unpack8(const uint32_t (&w)[7], uint32_t (&r)[8]) {
    r[0] = w[0] & RES_MASK;
    r[1] = __funnelshift_r(w[0], w[1], 28) & RES_MASK;
    r[2] = __funnelshift_r(w[1], w[2], 24) & RES_MASK;
    r[3] = __funnelshift_r(w[2], w[3], 20) & RES_MASK;
    r[4] = __funnelshift_r(w[3], w[4], 16) & RES_MASK;
    r[5] = __funnelshift_r(w[4], w[5], 12) & RES_MASK;
    r[6] = __funnelshift_r(w[5], w[6], 8) & RES_MASK;
    r[7] = w[6] >> 4;
}

__host__ __device__ __forceinline__ void pack8(const uint32_t (&r)[8], uint32_t (&w)[7]) {
    w[0] = r[0] | r[1] << 28;
    w[1] = r[1] >> 4 | r[2] << 24;
    w[2] = r[2] >> 8 | r[3] << 20;
    w[3] = r[3] >> 12 | r[4] << 16;
    w[4] = r[4] >> 16 | r[5] << 12;
    w[5] = r[5] >> 20 | r[6] << 8;
    w[6] = r[6] >> 24 | r[7] << 4;
}

// Residue m of a packed row (reads the second word only where the residue
// straddles two words, so never past the row).
__device__ __forceinline__ uint32_t unpack1(const uint32_t *row, int m) {
    const int bit = 28 * m, w = bit >> 5, sh = bit & 31;
    const uint32_t hi = sh > 4 ? row[w + 1] : 0u;
    return __funnelshift_r(row[w], hi, sh) & RES_MASK;
}

DbLayout make_db_layout(int T, int nu1, int nu2);

// Per-query descriptor: keys, workspace and database shape of one query.
// Kernels take an array of them (one per query of the launch), so queries
// against databases of different shapes can share a launch.
struct QDesc {
    // client keys, Montgomery form, [rows][cols][2][D]
    const uint32_t *left;    // [n_left][2][t_left]
    const uint32_t *right;   // [n_right][2][t_right]
    const uint32_t *conv;    // [2][2*t_conv]
    const uint32_t *pack;    // [n][n+1][t_conv]
    // workspace
    const uint32_t *query;   // [2][2][D] query ciphertext (round-0 input)
    uint32_t *v[2];          // expansion ping-pong [2^g][2][2][D]
    uint32_t *sel;           // [rows][D][4]  (row0 q1, row0 q2, row1 q1, row1 q2)
    uint32_t *gsw_in;        // [nu2*t_gsw][2][2][D]
    uint32_t *gsw;           // [nu2][2][2*t_gsw][2][D], Montgomery form
    uint32_t *acc;           // [T][cols][2][2][D]  DB-multiply output
    uint64_t *raw;           // [T][cols][2][D]     fold buffer
    uint8_t *resp;           // response bytes
    int nu1, nu2, g, stop, capture;
    int active;
};

struct StageParams {
    int n, T, pt_bits, q2_bits;
    int t_left, t_right, t_gsw, t_conv;
};


// Multiprocessor count of the current device.
int sm_count();

// One CTA whose barrier wait nothing completes: gives up after limit_ns and
// sets *err = 1 (the failure path of the multiply kernels' bounded waits).
cudaError_t launch_wait_probe(int *err, uint64_t limit_ns, cudaStream_t st);

// Checked mode: *bad = min(*bad, index of every region (address, length
// pairs) whose bytes are not all `fill`).
cudaError_t launch_check_guards(const uint64_t *regions, int n, uint8_t fill, uint32_t *bad, cudaStream_t st);

// Twiddle tables (device, one set per context).
void build_twiddles_host(TwiddleSet *host);

// raw u64[count][D] -> NTT u32[count][2][D] (canonical)
cudaError_t launch_to_ntt(const uint64_t *raw, uint32_t *out, int count, const TwiddleSet *tw,
                          cudaStream_t st);
// NTT u32[count][2][D] (values < 2p) -> raw u64[count][D]
cudaError_t launch_from_ntt(const uint32_t *in, uint64_t *raw, int count, const TwiddleSet *tw,
                            cudaStream_t st);
// Plain residue transforms in place: u32[count][2][D], canonical in/out;
// inverse includes the 2048^-1 scaling.
cudaError_t launch_ntt_planes(uint32_t *a, int count, bool inverse, const TwiddleSet *tw,
                              cudaStream_t st);
// automorphism x -> x^t on raw u64[count][D]
cudaError_t launch_automorph(const uint64_t *in, uint64_t *out, int count, uint32_t t,
                             cudaStream_t st);

// u8 records [rec_count][T][D] (record = row*cols + col) -> database image.
// `tmp` holds the chunk's NTT-form residues (rec_count * T * 2 * D u32).  A
// packed group (8 combos of a row) comes from 8 consecutive records (cols >= 8)
// or from one whole row (cols < 8), so rec_begin must be a multiple of 8 and
// rec_count too unless the chunk ends the database.
cudaError_t launch_db_encode(const uint8_t *records, uint64_t rec_begin, uint64_t rec_count,
                             int pt_bits, const DbLayout &L, uint32_t *tmp, uint32_t *db, const TwiddleSet *tw,
                             cudaStream_t st);
// NTT-form u32 planes [T][cols][rows][2][D] -> database image
cudaError_t launch_db_import(const uint32_t *planes, const DbLayout &L, uint32_t *db,
                             cudaStream_t st);

// First-dimension multiply for the `nq` queries qd[0..nq) against one
// database: reads qd[q].sel (u32[rows][D][4], row0 q1, row0 q2, row1 q1,
// row1 q2) and writes qd[q].acc (u32[T][cols][2 rows][2][D]), canonical.
// Streams the image once per query (bandwidth-bound variant).  With pdl,
// launched dependent on the previous kernel of the stream (programmatic
// dependent launch): its image stream starts before that kernel ends.
cudaError_t launch_db_mul(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                          cudaStream_t st, bool pdl = false);
// Same result, reading each database residue once per group of 8 queries
// on the integer pipe (compute-bound variant).
bool db_mul_batch_supported(const DbLayout &L);
cudaError_t launch_db_mul_batch(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, cudaStream_t st);

// Tensor-core variant (tcgen05, exact fp16 digit products): the selectors of
// up to TC_MAX_Q queries are first split into digit tiles in `limbs`
// (tc_limb_bytes(L) bytes); each unit of the image is then multiplied by them
// with fp32 accumulation in tensor memory, in launches over chunks of slots
// whose results pass through `out` (tc_out_bytes(L) bytes) on their way to
// the queries' accumulator planes.
constexpr int TC_MAX_Q = 32;
bool db_mul_tc_supported(const DbLayout &L);
uint64_t tc_limb_bytes(const DbLayout &L);
uint64_t tc_out_bytes(const DbLayout &L);
// kernels one launch_db_mul_tc call launches: the digit split, then a
// multiply and a transpose per chunk of slots
int tc_launches(const DbLayout &L);
cudaError_t launch_db_mul_tc(const uint32_t *db, const DbLayout &L, const QDesc *qd, int nq, uint8_t *limbs,
                             uint32_t *out, int *err, cudaStream_t st);

}  // namespace sp
