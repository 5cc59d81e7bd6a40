// Seed expansion of the uniform rows of a client's key matrices
// (csrc/seeded.cu).
#pragma once
#include <algorithm>

#include "kernels.cuh"

namespace sp {

struct SeedKey {
    uint32_t w[8];   // the 32-byte seed as little-endian words
};

// Where the row-0 polynomials of a key set live in the client key buffer
// (u32, Montgomery form): expansion-left [n_left][2][t_left][2][D], then
// expansion-right [n_right][2][t_right][2][D], conversion [2][2*t_conv][2][D],
// packing [n][n+1][t_conv][2][D].  Row-0 polynomial P counts left (r, j),
// right (r, j), conversion (j), packing (r, j).
struct SeedRowMap {
    int n_left, t_left, n_right, t_right, t_conv, n;
    uint32_t polys;   // n_left*t_left + n_right*t_right + 2*t_conv + n*t_conv
    __host__ __device__ uint64_t offset(uint32_t P) const;
};

cudaError_t launch_seed_rows(const SeedKey &key, const SeedRowMap &map, uint32_t *keys, cudaStream_t st);

}  // namespace sp
