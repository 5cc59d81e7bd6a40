/*
 * CPU oracle for the Spiral PIR server answer path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is compiled into
 * oracle/_build/liboracle.so and may be used only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * (the CUDA library under gpu-pir_gb300/) never links, loads or calls it.
 *
 * Everything here is exact modular integer arithmetic written for clarity,
 * not speed: residues are reduced with plain `%` after every product, so
 * the values it returns are canonical (in [0, p) per prime, [0, q) raw).
 *
 * Ring: Z_q[x]/(x^2048 + 1), q = q1*q2, q1 = 268369921, q2 = 249561089
 * (gpu-pir/params.cuh:25-31).  "NTT form" is the reference's spiral order:
 * the in-place Cooley-Tukey negacyclic transform with bit-reversed powers of
 * the primitive 4096-th root psi (gpu-pir/ntt_28bit.cuh:31-131,
 * gpu-pir/host.cu:64-71, gpu-pir/cpu_version/ntt.py:25-52,93-216).
 *
 * Layout conventions of this file (all little-endian, row-major):
 *   crt poly   u32[2][D]                 residues mod q1 then mod q2
 *   raw poly   u64[D]                    coefficients mod q
 *   NTT ct     u32[rows][2][D]           a Regev ciphertext has rows = 2
 *   raw ct     u64[rows][D]
 *   matrix     u32[rows][cols][2][D]     key matrices, GSW ciphertexts
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define D 2048
#define LOGD 11
#define MOD_BITS 56
typedef unsigned __int128 u128;

static const uint32_t QP[2] = {268369921u, 249561089u};
static const uint32_t PSI[2] = {66687u, 158221u};
static const uint64_t QQ = (uint64_t)268369921u * (uint64_t)249561089u;

static uint32_t tw_fwd[2][D];
static uint32_t tw_inv[2][D];
static uint32_t n_inv[2];
static uint32_t crt_m[2]; /* crt_m[0] = q2^-1 mod q1, crt_m[1] = q1^-1 mod q2 */

static uint32_t powmod(uint64_t b, uint64_t e, uint32_t p) {
    uint64_t r = 1;
    b %= p;
    while (e) {
        if (e & 1) r = r * b % p;
        b = b * b % p;
        e >>= 1;
    }
    return (uint32_t)r;
}

static uint32_t brev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

/* Twiddle tables: psi^brev11(i) and psi^-brev11(i) (gpu-pir/host.cu:64-71,
 * cpu_version/ntt.py:25-29), kept in plain (non-Montgomery) form. */
__attribute__((constructor)) static void or_init_tables(void) {
    for (int k = 0; k < 2; k++) {
        uint32_t p = QP[k];
        uint32_t psi_inv = powmod(PSI[k], 4095, p); /* psi^4096 = 1 */
        for (uint32_t i = 0; i < D; i++) {
            tw_fwd[k][i] = powmod(PSI[k], brev(i, LOGD), p);
            tw_inv[k][i] = powmod(psi_inv, brev(i, LOGD), p);
        }
        n_inv[k] = powmod(D, p - 2, p);
    }
    crt_m[0] = powmod(QP[1], QP[0] - 2, QP[0]);
    crt_m[1] = powmod(QP[0], QP[1] - 2, QP[1]);
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* R1/R2/R3: negacyclic NTT and inverse NTT                             */
/* ------------------------------------------------------------------ */

/* Forward transform of one residue plane, in place, canonical in and out.
 * Stage m (1, 2, 4, ..., 1024) pairs x[j] with x[j + h], h = 1024/m, and
 * block i uses psi^brev(m+i): the same butterfly schedule as
 * gpu-pir/ntt_28bit.cuh:44-129 (radix-8, shuffle and radix-8 phases all
 * apply this schedule) and cpu_version/ntt.py:93-199. */
void or_ntt_fwd(uint32_t *a, int k) {
    const uint64_t p = QP[k];
    for (int m = 1, h = D / 2; m < D; m <<= 1, h >>= 1) {
        for (int i = 0; i < m; i++) {
            const uint64_t s = tw_fwd[k][m + i];
            uint32_t *x = a + 2 * i * h;
            for (int j = 0; j < h; j++) {
                uint64_t u = x[j], v = (uint64_t)x[j + h] * s % p;
                x[j] = (uint32_t)((u + v) % p);
                x[j + h] = (uint32_t)((u + p - v) % p);
            }
        }
    }
}

/* Inverse transform (Gentleman-Sande, stages in reverse order) including
 * the 2048^-1 scaling.  gpu-pir/ntt_28bit.cuh:145-231 leaves the scaling
 * out and folds it into the inverse-CRT constants (params.cuh:33-35); the
 * value is the same once both are applied. */
void or_ntt_inv(uint32_t *a, int k) {
    const uint64_t p = QP[k];
    for (int m = D / 2, h = 1; m >= 1; m >>= 1, h <<= 1) {
        for (int i = 0; i < m; i++) {
            const uint64_t s = tw_inv[k][m + i];
            uint32_t *x = a + 2 * i * h;
            for (int j = 0; j < h; j++) {
                uint64_t u = x[j], v = x[j + h];
                x[j] = (uint32_t)((u + v) % p);
                x[j + h] = (uint32_t)((u + p - v) * s % p);
            }
        }
    }
    for (int i = 0; i < D; i++) a[i] = (uint32_t)((uint64_t)a[i] * n_inv[k] % p);
}

/* Inverse CRT of one coefficient (gpu-pir/arith.cuh:51-59). */
static inline uint64_t crt_join(uint32_t a, uint32_t b) {
    uint64_t x1 = (uint64_t)a * crt_m[0] % QP[0];
    uint64_t x2 = (uint64_t)b * crt_m[1] % QP[1];
    u128 s = (u128)x1 * QP[1] + (u128)x2 * QP[0];
    return (uint64_t)(s % QQ);
}

/* NTT form -> raw (gpu-pir/gadget.cuh:8-24 from_ntt_regs: INTT per prime,
 * then inverse CRT). */
void or_from_ntt(const uint32_t *in, uint64_t *out) {
    uint32_t t0[D], t1[D];
    memcpy(t0, in, sizeof t0);
    memcpy(t1, in + D, sizeof t1);
    or_ntt_inv(t0, 0);
    or_ntt_inv(t1, 1);
    for (int i = 0; i < D; i++) out[i] = crt_join(t0[i], t1[i]);
}

/* raw -> NTT form (gpu-pir/classes.cuh:140-174 to_ntt). */
void or_to_ntt(const uint64_t *in, uint32_t *out) {
    for (int k = 0; k < 2; k++) {
        for (int i = 0; i < D; i++) out[k * D + i] = (uint32_t)(in[i] % QP[k]);
        or_ntt_fwd(out + k * D, k);
    }
}

void or_ntt_fwd_many(uint32_t *a, uint64_t count) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++) {
        or_ntt_fwd(a + (size_t)i * 2 * D, 0);
        or_ntt_fwd(a + (size_t)i * 2 * D + D, 1);
    }
}

void or_from_ntt_many(const uint32_t *in, uint64_t *out, uint64_t count) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++)
        or_from_ntt(in + (size_t)i * 2 * D, out + (size_t)i * D);
}

void or_to_ntt_many(const uint64_t *in, uint32_t *out, uint64_t count) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; i++)
        or_to_ntt(in + (size_t)i * D, out + (size_t)i * 2 * D);
}

/* ------------------------------------------------------------------ */
/* R7: automorphism x -> x^t on raw coefficients                        */
/* ------------------------------------------------------------------ */

/* gpu-pir/automorph.cuh:28-50 and automorph_test.cu:14-22: coefficient i
 * moves to (i*t mod D) and is negated when floor(i*t / D) is odd.  The
 * reference writes MODULUS - 0 = q for a zero coefficient; the canonical
 * value 0 is used here. */
void or_automorph(const uint64_t *in, uint64_t *out, uint32_t t) {
    for (uint32_t i = 0; i < D; i++) {
        uint64_t it = (uint64_t)i * t;
        uint32_t idx = (uint32_t)(it % D);
        uint64_t v = in[i];
        out[idx] = ((it / D) & 1) ? (v ? QQ - v : 0) : v;
    }
}

/* ------------------------------------------------------------------ */
/* R8: gadget decomposition and gadget product                          */
/* ------------------------------------------------------------------ */

/* Digit width for a gadget of length t: ceil(56 / t)
 * (gpu-pir/gadget.cuh:37-39, cpu_version/gadget.py:35-36). */
int or_bits_per(int t) { return (MOD_BITS + t - 1) / t; }

/* acc[r] += sum_{j<rdim, k<t} mat[r][j + k*rdim] * NTT(digit_k(rows[j]))
 * for r < out_rows, all in NTT form mod each prime.  Unsigned digits
 * (x >> k*bits) & mask, row index j + k*rdim: gpu-pir/gadget.cuh:55-82,
 * cpu_version/gadget.py:52-79.  `mat` is u32[out_rows][rdim*t][2][D]. */
static void gadget_mac(const uint64_t *rows, int rdim, int t, const uint32_t *mat,
                       int out_rows, uint32_t *acc) {
    const int bits = or_bits_per(t);
    const uint64_t mask = (bits >= 64) ? ~0ull : ((1ull << bits) - 1);
    const int cols = rdim * t;
    uint32_t dig[2 * D];
    for (int j = 0; j < rdim; j++) {
        for (int k = 0; k < t; k++) {
            const int col = j + k * rdim;
            const int shift = k * bits;
            for (int i = 0; i < D; i++) {
                uint64_t d = shift < 64 ? (rows[(size_t)j * D + i] >> shift) & mask : 0;
                dig[i] = (uint32_t)(d % QP[0]);
                dig[D + i] = (uint32_t)(d % QP[1]);
            }
            or_ntt_fwd(dig, 0);
            or_ntt_fwd(dig + D, 1);
            for (int r = 0; r < out_rows; r++) {
                const uint32_t *m = mat + ((size_t)r * cols + col) * 2 * D;
                uint32_t *a = acc + (size_t)r * 2 * D;
                for (int kk = 0; kk < 2; kk++)
                    for (int i = 0; i < D; i++) {
                        uint64_t v = (uint64_t)m[kk * D + i] * dig[kk * D + i] % QP[kk];
                        a[kk * D + i] = (uint32_t)((a[kk * D + i] + v) % QP[kk]);
                    }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* R6: coefficient expansion                                            */
/* ------------------------------------------------------------------ */

static int ceil_log2(uint64_t x) {
    int v = 0;
    uint64_t p = 1;
    while (p < x) { p <<= 1; v++; }
    return v;
}

/* g = ceil(log2(t_gsw*nu2 + 2^nu1)), stop_round = ceil(log2(t_gsw*nu2))
 * (gpu-pir/expansion.cuh:83-85). */
int or_expansion_g(int nu1, int nu2, int t_gsw) {
    return ceil_log2((uint64_t)t_gsw * nu2 + (1ull << nu1));
}
int or_expansion_stop(int nu2, int t_gsw) { return ceil_log2((uint64_t)t_gsw * nu2); }

/* NTT form of x^(-2^r) = -x^(D - 2^r): multiplier of the second half of
 * round r (gpu-pir/expansion.cuh:171-211 v_neg1). */
void or_neg1(int r, uint32_t *out) {
    uint64_t raw[D];
    memset(raw, 0, sizeof raw);
    raw[D - (1u << r)] = QQ - 1;
    or_to_ntt(raw, out);
}

/* One expansion action on v_i in place (gpu-pir/expansion.cuh:87-166):
 *   c = raw(v_i); c' = tau_t(c)
 *   v_i += [0; NTT(c'.row1)] + W * NTT(G^-1(c'.row0))
 * with the unsigned t_w-digit gadget of W (rdim 1). */
static void expand_action(uint32_t *v, const uint32_t *w, int t_w, uint32_t t_auto) {
    uint64_t raw[2][D], aut[2][D];
    or_from_ntt(v, raw[0]);
    or_from_ntt(v + 2 * D, raw[1]);
    or_automorph(raw[0], aut[0], t_auto);
    or_automorph(raw[1], aut[1], t_auto);
    uint32_t acc[2 * 2 * D];
    memset(acc, 0, sizeof acc);
    gadget_mac(aut[0], 1, t_w, w, 2, acc);
    uint32_t b[2 * D];
    or_to_ntt(aut[1], b);
    for (int kk = 0; kk < 2; kk++)
        for (int i = 0; i < D; i++) {
            uint64_t p = QP[kk];
            uint32_t *a0 = v + kk * D, *a1 = v + 2 * D + kk * D;
            a0[i] = (uint32_t)(((uint64_t)a0[i] + acc[kk * D + i]) % p);
            a1[i] = (uint32_t)(((uint64_t)a1[i] + acc[2 * D + kk * D + i] + b[kk * D + i]) % p);
        }
}

/* Coefficient expansion of one query ciphertext (NTT form) into
 * v[0 .. 2^rounds) (u32[2^rounds][2][2][D], NTT form).
 *   left:  u32[>= rounds][2][t_left][2][D]
 *   right: u32[>= stop+1][2][t_right][2][D]
 * Round r: v[i + 2^r] = x^(-2^r) v[i] for i < 2^r, then the expansion
 * action on every live i < 2^(r+1); odd i use right[r], even i use left[r]
 * except in round 0 (right[0]); odd i are pruned past stop_round and at
 * stop_round when i/2 >= t_gsw*nu2 (gpu-pir/expansion.cuh:87-130,
 * expansion.cuh:171-259).  `rounds` is g for a full expansion; the
 * one-round golden vector uses rounds = 1. */
void or_expand(const uint32_t *query, const uint32_t *left, int t_left, const uint32_t *right,
               int t_right, int nu1, int nu2, int t_gsw, int rounds, uint32_t *v) {
    const size_t ct = 2 * 2 * D;
    const int stop = or_expansion_stop(nu2, t_gsw);
    const uint64_t max_bits = (uint64_t)t_gsw * nu2;
    memset(v, 0, ((size_t)1 << rounds) * ct * sizeof(uint32_t));
    memcpy(v, query, ct * sizeof(uint32_t));
    for (int r = 0; r < rounds; r++) {
        const uint64_t num_in = 1ull << r;
        uint32_t neg1[2 * D];
        or_neg1(r, neg1);
        for (uint64_t i = 0; i < num_in; i++)
            for (int row = 0; row < 2; row++)
                for (int kk = 0; kk < 2; kk++)
                    for (int z = 0; z < D; z++) {
                        const uint32_t *src = v + i * ct + row * 2 * D + kk * D;
                        uint32_t *dst = v + (i + num_in) * ct + row * 2 * D + kk * D;
                        dst[z] = (uint32_t)((uint64_t)src[z] * neg1[kk * D + z] % QP[kk]);
                    }
        const uint32_t t_auto = (D >> r) + 1;
        #pragma omp parallel for schedule(dynamic, 1)
        for (int64_t ii = 0; ii < (int64_t)(2 * num_in); ii++) {
            const uint64_t i = (uint64_t)ii;
            if (stop > 0 && r > stop && (i & 1)) continue;
            if (stop > 0 && r == stop && (i & 1) && (i / 2) >= max_bits) continue;
            const int use_left = (r != 0) && ((i & 1) == 0);
            const uint32_t *w = use_left ? left + (size_t)r * 2 * t_left * 2 * D
                                         : right + (size_t)r * 2 * t_right * 2 * D;
            expand_action(v + i * ct, w, use_left ? t_left : t_right, t_auto);
        }
    }
}

/* ------------------------------------------------------------------ */
/* R9: Regev -> GSW conversion,  R10: GSW negation                      */
/* ------------------------------------------------------------------ */

/* For each of nu2 dimensions build a 2 x 2*t_gsw GSW ciphertext from the
 * t_gsw Regev encodings of (bit * 2^(bits*j)): column 2j+1 is the Regev
 * ciphertext itself, column 2j is V * NTT(G^-1_{2,t_conv}(raw(c)))
 * (the conversion slot of gpu-pir/structures.cuh:173-177 and the fold
 * gadget layout of gpu-pir/folding.cuh:9-27; the reference leaves the
 * procedure as a stub, cpu_version/conversion.py:3, and it follows the
 * Spiral paper's Regev-to-GSW step).
 *   regev: u32[nu2*t_gsw][2][2][D]   conv: u32[2][2*t_conv][2][D]
 *   gsw:   u32[nu2][2][2*t_gsw][2][D] */
void or_regev_to_gsw(const uint32_t *regev, const uint32_t *conv, int nu2, int t_gsw, int t_conv,
                     uint32_t *gsw) {
    const size_t P = 2 * D;
    const int cols = 2 * t_gsw;
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t idx = 0; idx < (int64_t)nu2 * t_gsw; idx++) {
        const int i = (int)(idx / t_gsw), j = (int)(idx % t_gsw);
        const uint32_t *c = regev + (size_t)idx * 2 * P;
        uint32_t *g = gsw + (size_t)i * 2 * cols * P;
        for (int row = 0; row < 2; row++)
            memcpy(g + ((size_t)row * cols + 2 * j + 1) * P, c + row * P, P * sizeof(uint32_t));
        uint64_t raw[2][D];
        or_from_ntt(c, raw[0]);
        or_from_ntt(c + P, raw[1]);
        uint32_t acc[2 * 2 * D];
        memset(acc, 0, sizeof acc);
        gadget_mac(&raw[0][0], 2, t_conv, conv, 2, acc);
        for (int row = 0; row < 2; row++)
            memcpy(g + ((size_t)row * cols + 2 * j) * P, acc + row * P, P * sizeof(uint32_t));
    }
}

/* Vneg = G - V in NTT form, G = I_2 (x) (1, 2^b, ..., 2^(b(t-1))) with
 * column c = j + 2k holding 2^(b k) on row j (the relation between
 * test_data/client_folding_keys.dat and client_folding_keys_neg.dat; the
 * reference's cpu_version/folding.py:7-12 is a stub).  The NTT of a
 * constant is that constant in every slot.  gsw: u32[count][2][2t][2][D]. */
void or_gsw_neg(const uint32_t *gsw, int count, int t, uint32_t *neg) {
    const int bits = or_bits_per(t);
    const int cols = 2 * t;
    for (int c = 0; c < count; c++)
        for (int row = 0; row < 2; row++)
            for (int col = 0; col < cols; col++)
                for (int kk = 0; kk < 2; kk++) {
                    const uint64_t p = QP[kk];
                    const int k = col / 2;
                    uint64_t gval = ((col & 1) == row && bits * k < 64) ? ((1ull << (bits * k)) % p) : 0;
                    size_t off = ((((size_t)c * 2 + row) * cols + col) * 2 + kk) * D;
                    for (int z = 0; z < D; z++)
                        neg[off + z] = (uint32_t)((gval + p - gsw[off + z]) % p);
                }
}

/* ------------------------------------------------------------------ */
/* R5/R11: database encoding and first-dimension multiply               */
/* ------------------------------------------------------------------ */

/* Encode plaintext records into NTT form.  Record index i = row*2^nu2 + col
 * (row: first dimension, col: folded dimension); a record is n*n
 * polynomials of D coefficients in [0, 2^pt_bits), one byte each when
 * pt_bits <= 8.  Each coefficient is recentred to (-p/2, p/2] mod q before
 * the NTT.  Output layout (the reference's Database<Poly<u32>> struct,
 * gpu-pir/structures.cuh:200-210, with the n*n index outermost):
 *   db: u32[n*n][2^nu2 cols][2^nu1 rows][2][D]. */
void or_db_encode(const uint8_t *records, int n, int nu1, int nu2, int pt_bits, uint32_t *db) {
    const uint64_t rows = 1ull << nu1, cols = 1ull << nu2;
    const int T = n * n;
    const uint64_t pmod = 1ull << pt_bits;
    #pragma omp parallel for schedule(static)
    for (int64_t rec = 0; rec < (int64_t)(rows * cols); rec++) {
        const uint64_t row = (uint64_t)rec / cols, col = (uint64_t)rec % cols;
        for (int t = 0; t < T; t++) {
            const uint8_t *src = records + ((size_t)rec * T + t) * D;
            uint64_t raw[D];
            for (int z = 0; z < D; z++) {
                uint64_t v = src[z];
                raw[z] = (v > pmod / 2) ? QQ - (pmod - v) : v;
            }
            or_to_ntt(raw, db + ((((size_t)t * cols + col) * rows + row) * 2) * D);
        }
    }
}

/* acc[t][col][ct_row] = sum_row sel[row][ct_row] * db[t][col][row], per
 * prime and NTT slot, accumulated in 128 bits and reduced once
 * (gpu-pir/db_mul_test.cu:240-282 CPU loop; gpu-pir/db_mul.cuh:26-70).
 *   sel: u32[2^nu1][2][2][D]   acc: u32[T][2^nu2][2][2][D] */
void or_db_mul(const uint32_t *db, const uint32_t *sel, int T, int nu1, int nu2, uint32_t *acc) {
    const uint64_t rows = 1ull << nu1, cols = 1ull << nu2;
    #pragma omp parallel for schedule(static)
    for (int64_t tc = 0; tc < (int64_t)(T * cols); tc++) {
        const uint64_t t = (uint64_t)tc / cols, col = (uint64_t)tc % cols;
        for (int kk = 0; kk < 2; kk++) {
            for (int z = 0; z < D; z++) {
                u128 a0 = 0, a1 = 0;
                for (uint64_t row = 0; row < rows; row++) {
                    uint64_t dv = db[((((t * cols + col) * rows + row) * 2) + kk) * D + z];
                    a0 += (u128)((uint64_t)sel[((row * 2 + 0) * 2 + kk) * D + z] * dv);
                    a1 += (u128)((uint64_t)sel[((row * 2 + 1) * 2 + kk) * D + z] * dv);
                }
                size_t o = (((t * cols + col) * 2) * 2 + kk) * D + z;
                acc[o] = (uint32_t)(a0 % QP[kk]);
                acc[o + 2 * D] = (uint32_t)(a1 % QP[kk]);
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* R12: GSW folding                                                     */
/* ------------------------------------------------------------------ */

/* Fold 2^nu2 raw ciphertexts down to cts[0] (gpu-pir/folding.cuh:9-53,
 * cpu_version/folding.py:19-45):
 *   for level d: num_per /= 2; for i < num_per:
 *     cts[i] = raw( G^-1(cts[num_per+i]) . V[nu2-1-d]
 *                 + G^-1(cts[i]) . Vneg[nu2-1-d] )
 *   cts: u64[2^nu2][2][D] (in place)   V, Vneg: u32[nu2][2][2t][2][D] */
void or_fold(uint64_t *cts, const uint32_t *V, const uint32_t *Vneg, int nu2, int t_gsw) {
    const size_t gsw_sz = (size_t)2 * 2 * t_gsw * 2 * D;
    uint64_t num_per = 1ull << nu2;
    for (int d = 0; d < nu2; d++) {
        num_per >>= 1;
        const uint32_t *v = V + (size_t)(nu2 - 1 - d) * gsw_sz;
        const uint32_t *vn = Vneg + (size_t)(nu2 - 1 - d) * gsw_sz;
        #pragma omp parallel for schedule(dynamic, 1)
        for (int64_t i = 0; i < (int64_t)num_per; i++) {
            uint32_t acc[2 * 2 * D];
            memset(acc, 0, sizeof acc);
            gadget_mac(cts + (num_per + i) * 2 * D, 2, t_gsw, v, 2, acc);
            gadget_mac(cts + i * 2 * D, 2, t_gsw, vn, 2, acc);
            or_from_ntt(acc, cts + i * 2 * D);
            or_from_ntt(acc + 2 * D, cts + i * 2 * D + D);
        }
    }
}

/* Fold for T independent instances: cts u64[T][2^nu2][2][D]; result of
 * instance t in cts[t][0]. */
void or_fold_many(uint64_t *cts, int T, const uint32_t *V, const uint32_t *Vneg, int nu2, int t_gsw) {
    for (int t = 0; t < T; t++)
        or_fold(cts + ((size_t)t << nu2) * 2 * D, V, Vneg, nu2, t_gsw);
}

/* ------------------------------------------------------------------ */
/* R14: packing, modulus switching and serialisation                    */
/* ------------------------------------------------------------------ */

/* Pack n*n raw Regev ciphertexts (index r*n + c) into one (n+1) x n
 * matrix-Regev ciphertext, returned raw:
 *   column c = sum_r  W_r * NTT(G^-1_{t_conv}(ct[r*n+c].row0))
 *                   + e_{1+r} * NTT(ct[r*n+c].row1)
 * with W_r: u32[n+1][t_conv][2][D] (the response packing of the Spiral
 * paper; absent from the reference).
 *   cts: u64[n*n][2][D]   keys: u32[n][n+1][t_conv][2][D]
 *   out: u64[n+1][n][D] */
void or_pack(const uint64_t *cts, const uint32_t *keys, int n, int t_conv, uint64_t *out) {
    const size_t P = 2 * D;
    const size_t key_sz = (size_t)(n + 1) * t_conv * P;
    uint32_t *acc = (uint32_t *)calloc((size_t)(n + 1) * P, sizeof(uint32_t));
    for (int c = 0; c < n; c++) {
        memset(acc, 0, (size_t)(n + 1) * P * sizeof(uint32_t));
        for (int r = 0; r < n; r++) {
            const uint64_t *ct = cts + (size_t)(r * n + c) * 2 * D;
            gadget_mac(ct, 1, t_conv, keys + (size_t)r * key_sz, n + 1, acc);
            uint32_t b[2 * D];
            or_to_ntt(ct + D, b);
            for (int kk = 0; kk < 2; kk++)
                for (int z = 0; z < D; z++) {
                    uint32_t *a = acc + (size_t)(1 + r) * P + kk * D;
                    a[z] = (uint32_t)(((uint64_t)a[z] + b[kk * D + z]) % QP[kk]);
                }
        }
        for (int row = 0; row <= n; row++)
            or_from_ntt(acc + (size_t)row * P, out + ((size_t)row * n + c) * D);
    }
    free(acc);
}

/* Rescale x in Z_q (centred) to Z_{q'}: round(x * q' / q) mod q', ties
 * away from zero. */
uint64_t or_rescale(uint64_t x, uint64_t q_in, uint64_t q_out) {
    x %= q_in;
    if (x >= (q_in + 1) / 2) {
        u128 num = (u128)(q_in - x) * q_out + q_in / 2;
        uint64_t y = (uint64_t)(num / q_in) % q_out;
        return y ? q_out - y : 0;
    }
    u128 num = (u128)x * q_out + q_in / 2;
    return (uint64_t)(num / q_in) % q_out;
}

uint64_t or_response_bytes(int n, int pt_bits, int q2_bits) {
    uint64_t bits = (uint64_t)n * D * q2_bits + (uint64_t)n * n * D * (pt_bits + 2);
    return (bits + 63) / 64 * 8;
}

/* Modulus-switch the packed ciphertext and serialise it: first row (n
 * polys) rescaled to 2^q2_bits, the other n rows (n*n polys) to 4p, each
 * value written little-endian-bit-first at consecutive bit offsets, total
 * rounded up to 64 bits.  packed: u64[n+1][n][D] raw. */
void or_encode_response(const uint64_t *packed, int n, int pt_bits, int q2_bits, uint8_t *out) {
    const uint64_t q2 = 1ull << q2_bits;
    const int q1_bits = pt_bits + 2;
    const uint64_t q1 = 1ull << q1_bits;
    memset(out, 0, or_response_bytes(n, pt_bits, q2_bits));
    uint64_t off = 0;
    const uint64_t total = (uint64_t)(n + 1) * n * D;
    for (uint64_t i = 0; i < total; i++) {
        const int nb = (i < (uint64_t)n * D) ? q2_bits : q1_bits;
        const uint64_t v = or_rescale(packed[i], QQ, (i < (uint64_t)n * D) ? q2 : q1);
        for (int b = 0; b < nb; b++, off++)
            if ((v >> b) & 1) out[off >> 3] |= (uint8_t)(1u << (off & 7));
    }
}

/* ------------------------------------------------------------------ */
/* Full answer                                                          */
/* ------------------------------------------------------------------ */

/* Answer one query against an encoded database (or_db_encode layout):
 * expand -> split -> Regev-to-GSW -> G - V -> first-dimension multiply ->
 * raw -> fold -> pack -> modulus switch.  Optional outputs (may be NULL):
 * expanded u32[2^g][2][2][D], acc (DB-multiply output, or_db_mul layout),
 * folded u64[n*n][2][D]. */
int or_answer(const uint32_t *db, int n, int nu1, int nu2, int pt_bits, int q2_bits, int t_left,
              int t_right, int t_gsw, int t_conv, const uint32_t *query, const uint32_t *left,
              const uint32_t *right, const uint32_t *conv, const uint32_t *pack_keys,
              uint8_t *response, uint32_t *expanded_out, uint32_t *acc_out, uint64_t *folded_out) {
    const size_t P = 2 * D, CT = 2 * P;
    const int g = or_expansion_g(nu1, nu2, t_gsw);
    const int T = n * n;
    const uint64_t rows = 1ull << nu1, cols = 1ull << nu2;
    uint32_t *v = (uint32_t *)malloc(((size_t)1 << g) * CT * sizeof(uint32_t));
    uint32_t *sel = (uint32_t *)malloc(rows * CT * sizeof(uint32_t));
    uint32_t *regev = (uint32_t *)malloc((size_t)nu2 * t_gsw * CT * sizeof(uint32_t));
    const size_t gsw_sz = (size_t)2 * 2 * t_gsw * P;
    uint32_t *gsw = (uint32_t *)malloc(nu2 * gsw_sz * sizeof(uint32_t));
    uint32_t *gneg = (uint32_t *)malloc(nu2 * gsw_sz * sizeof(uint32_t));
    uint32_t *acc = (uint32_t *)malloc((size_t)T * cols * CT * sizeof(uint32_t));
    uint64_t *raw = (uint64_t *)malloc((size_t)T * cols * 2 * D * sizeof(uint64_t));
    uint64_t *folded = (uint64_t *)malloc((size_t)T * 2 * D * sizeof(uint64_t));
    uint64_t *packed = (uint64_t *)malloc((size_t)(n + 1) * n * D * sizeof(uint64_t));
    if (!v || !sel || !regev || !gsw || !gneg || !acc || !raw || !folded || !packed) return -1;

    or_expand(query, left, t_left, right, t_right, nu1, nu2, t_gsw, g, v);
    for (uint64_t r = 0; r < rows; r++) memcpy(sel + r * CT, v + (2 * r) * CT, CT * 4);
    for (int i = 0; i < nu2 * t_gsw; i++) memcpy(regev + i * CT, v + (2 * (size_t)i + 1) * CT, CT * 4);
    or_regev_to_gsw(regev, conv, nu2, t_gsw, t_conv, gsw);
    or_gsw_neg(gsw, nu2, t_gsw, gneg);
    or_db_mul(db, sel, T, nu1, nu2, acc);
    or_from_ntt_many(acc, raw, (uint64_t)T * cols * 2);
    for (int t = 0; t < T; t++) {
        uint64_t *inst = raw + ((size_t)t * cols) * 2 * D;
        or_fold(inst, gsw, gneg, nu2, t_gsw);
        memcpy(folded + (size_t)t * 2 * D, inst, 2 * D * sizeof(uint64_t));
    }
    or_pack(folded, pack_keys, n, t_conv, packed);
    if (response) or_encode_response(packed, n, pt_bits, q2_bits, response);
    if (expanded_out) memcpy(expanded_out, v, ((size_t)1 << g) * CT * 4);
    if (acc_out) memcpy(acc_out, acc, (size_t)T * cols * CT * 4);
    if (folded_out) memcpy(folded_out, folded, (size_t)T * 2 * D * 8);
    free(v); free(sel); free(regev); free(gsw); free(gneg); free(acc); free(raw); free(folded); free(packed);
    return 0;
}
