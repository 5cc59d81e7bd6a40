// Kernel launchers of the Spiral answer path (host side declarations).
// Every launcher enqueues on `st` and returns the launch status.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sp {

// Tiled device layout of one database (packed u64 = residue q1 | residue q2 << 32):
//   [z_tile][col_group][row][t][c][z_in_tile]
// z_tile = z / ZT, col = col_group*cg + c, t < T (plaintext polynomial of the
// record).  A (z_tile, col_group) pair is one contiguous stream of
// rows * T*cg*ZT words, consumed front to back by one CTA of the multiply.
struct DbLayout {
    int T;        // n*n
    int nu1, nu2;
    int rows, cols;
    int cg;       // columns per group
    int ncg;      // cols / cg
    int zt;       // z tile (64)
    int nzt;      // D / zt
    uint64_t words;  // total u64 words
    __host__ __device__ uint64_t offset(int t, int row, int col, int z) const {
        int zti = z / zt, zi = z % zt, g = col / cg, c = col % cg;
        return ((((uint64_t)(zti * ncg + g) * rows + row) * T + t) * cg + c) * zt + zi;
    }
};

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
    uint32_t *ms;            // [n+1][n][D]         modulus-switched response
    uint8_t *resp;           // response bytes
    int nu1, nu2, g, stop, capture;
    int active;
};

struct StageParams {
    int n, T, pt_bits, q2_bits;
    int t_left, t_right, t_gsw, t_conv;
};


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

// u8 records [n_rec][T][D] (record = row*cols + col) -> tiled database image
cudaError_t launch_db_encode(const uint8_t *records, uint64_t rec_begin, uint64_t rec_count,
                             int pt_bits, const DbLayout &L, uint64_t *db, const TwiddleSet *tw,
                             cudaStream_t st);
// NTT-form u32 planes [T][cols][rows][2][D] -> tiled image
cudaError_t launch_db_import(const uint32_t *planes, const DbLayout &L, uint64_t *db,
                             cudaStream_t st);

// First-dimension multiply for the `nq` queries qd[0..nq) against one
// database: reads qd[q].sel (u32[rows][D][4], row0 q1, row0 q2, row1 q1,
// row1 q2) and writes qd[q].acc (u32[T][cols][2 rows][2][D]), canonical.
cudaError_t launch_db_mul(const uint64_t *db, const DbLayout &L, const QDesc *qd, int nq, int *err,
                          cudaStream_t st);
int db_mul_ctas(const DbLayout &L);
// Same result as launch_db_mul for nq > 1 queries, reading each database
// word once per group of 4 queries (compute-bound variant).
bool db_mul_batch_supported(const DbLayout &L);
cudaError_t launch_db_mul_batch(const uint64_t *db, const DbLayout &L, const QDesc *qd, int nq, cudaStream_t st);

}  // namespace sp
