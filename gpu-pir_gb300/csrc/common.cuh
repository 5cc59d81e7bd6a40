// Device-side building blocks of the Spiral answer path on GB300 (sm_103a).
//
// Ring Z_q[x]/(x^2048 + 1), q = q1*q2 with q1 = 268369921, q2 = 249561089
// (gpu-pir/params.cuh:25-31).  NTT form is the reference's "spiral order":
// the in-place Cooley-Tukey negacyclic transform with bit-reversed powers of
// psi (gpu-pir/ntt_28bit.cuh:31-131, gpu-pir/host.cu:64-71).
//
// One residue plane (2048 values mod one prime) is transformed by a group of
// 128 threads holding 16 values each, in three register phases separated by
// two shared-memory transposes:
//   layout A: thread t holds e = t + 128*j        stages h = 1024 .. 128
//   layout B: thread t holds e = 128*(t>>3) + (t&7) + 8*j   h = 64 .. 8
//   layout C: thread t holds e = 16*t + j         stages h = 4, 2, 1
// Raw-domain work (digits, inverse CRT) uses layout A (coalesced), NTT-domain
// work (key products) uses layout C (16 consecutive slots per thread).
// Digit transforms (inputs below 2^19 or p) skip the per-butterfly
// reduction and reduce once or twice per transform (ntt_fwd<LAZY>).
// Other butterflies are Harvey's lazy butterflies with Shoup products (values < 4p
// forward, < 2p inverse); the transposes use an XOR swizzle that is
// bank-conflict free for all three layouts.  Both directions read one
// twiddle table per prime: the inverse twiddle of block i at the stage with
// m blocks, psi^-brev11(m+i), equals -psi^brev11(2m-1-i) (psi^2048 = -1), so
// the inverse transform reads the forward entry 2m-1-i and folds the sign
// into its butterfly.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace sp {

constexpr int D = 2048;
constexpr int LOGD = 11;
constexpr uint32_t QP0 = 268369921u;
constexpr uint32_t QP1 = 249561089u;
constexpr uint64_t QQ = (uint64_t)QP0 * (uint64_t)QP1;
constexpr int MOD_BITS = 56;
constexpr int GROUP = 128;          // threads per NTT group
constexpr int VPT = D / GROUP;      // values per thread (16)

// ---------------------------------------------------------------- host math
constexpr uint32_t inv32(uint32_t p) {  // p^-1 mod 2^32 (Newton)
    uint32_t x = p;
    for (int i = 0; i < 5; i++) x *= 2u - p * x;
    return x;
}
constexpr uint64_t powmod_c(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1;
    b %= m;
    while (e) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
        e >>= 1;
    }
    return r;
}

struct Prime {
    uint32_t p;
    uint32_t pinv;      // p^-1 mod 2^32
    uint32_t r2;        // 2^64 mod p (to Montgomery form)
    uint32_t ninv_m;    // 2048^-1 * 2^32 mod p
    uint32_t crt_m;     // (other prime)^-1 * 2048^-1 * 2^32 mod p
    uint32_t two32;     // 2^32 mod p
};

constexpr Prime make_prime(uint32_t p, uint32_t other) {
    Prime c{};
    c.p = p;
    c.pinv = inv32(p);
    c.two32 = (uint32_t)((1ull << 32) % p);
    c.r2 = (uint32_t)((uint64_t)c.two32 * c.two32 % p);
    uint64_t ninv = powmod_c(D, p - 2, p);
    c.ninv_m = (uint32_t)(ninv * c.two32 % p);
    uint64_t oinv = powmod_c(other % p, p - 2, p);
    c.crt_m = (uint32_t)(oinv * ninv % p * c.two32 % p);
    return c;
}

constexpr Prime PRIME0_H = make_prime(QP0, QP1);
constexpr Prime PRIME1_H = make_prime(QP1, QP0);
// scalar copies (usable in device code)
constexpr uint32_t P0_PINV = PRIME0_H.pinv, P1_PINV = PRIME1_H.pinv;
constexpr uint32_t P0_R2 = PRIME0_H.r2, P1_R2 = PRIME1_H.r2;
constexpr uint32_t P0_NINV = PRIME0_H.ninv_m, P1_NINV = PRIME1_H.ninv_m;
constexpr uint32_t P0_CRT = PRIME0_H.crt_m, P1_CRT = PRIME1_H.crt_m;
constexpr uint32_t P0_TWO32 = PRIME0_H.two32, P1_TWO32 = PRIME1_H.two32;

__host__ __device__ __forceinline__ Prime prime_of(int k) {
    Prime c;
    c.p = k ? QP1 : QP0;
    c.pinv = k ? P1_PINV : P0_PINV;
    c.r2 = k ? P1_R2 : P0_R2;
    c.ninv_m = k ? P1_NINV : P0_NINV;
    c.crt_m = k ? P1_CRT : P0_CRT;
    c.two32 = k ? P1_TWO32 : P0_TWO32;
    return c;
}

// ------------------------------------------------------------ device math
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    // a < 2^32, b < p  ->  a*b*2^-32 mod p in (0, 2p)
    uint64_t u = (uint64_t)a * b;
    uint32_t m = (uint32_t)u * pinv;
    return (uint32_t)(u >> 32) - __umulhi(m, p) + p;
}

__device__ __forceinline__ uint32_t reduce2(uint32_t x, uint32_t twop) {  // [0,2*twop) -> [0,twop)
    return min(x, x - twop);
}

__device__ __forceinline__ uint32_t canon4(uint32_t x, uint32_t p) {  // [0,4p) -> [0,p)
    x = min(x, x - 2 * p);
    return min(x, x - p);
}

// x (< 2^56 or any u64 < p*2^32) mod p, canonical
__device__ __forceinline__ uint32_t mod_u64(uint64_t x, const Prime &c) {
    uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    // x*2^-32 mod p via Montgomery reduction of (hi:lo)
    uint32_t m = lo * c.pinv;
    uint32_t r = hi - __umulhi(m, c.p) + c.p;       // (0, 2p) when hi < p
    r = mont_mul(r, c.r2, c.p, c.pinv);             // * 2^64 * 2^-32 -> x
    return min(r, r - c.p);
}

// Inverse CRT of unscaled INTT outputs a0 (mod q1) and a1 (mod q2), both in
// [0, 2p): returns x in [0, q) with x = 2048^-1 * CRT(a0, a1).
__device__ __forceinline__ uint64_t icrt(uint32_t a0, uint32_t a1) {
    uint32_t x0 = mont_mul(a0, P0_CRT, QP0, P0_PINV);
    x0 = min(x0, x0 - QP0);
    uint32_t x1 = mont_mul(a1, P1_CRT, QP1, P1_PINV);
    x1 = min(x1, x1 - QP1);
    uint64_t s = (uint64_t)x0 * QP1 + (uint64_t)x1 * QP0;
    return s >= QQ ? s - QQ : s;
}

// ------------------------------------------------------------- barriers
__device__ __forceinline__ void group_sync(int bar_id) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "n"(GROUP) : "memory");
}

// -------------------------------------------------------------- swizzle
// Bank of element e: bits (e0^e5, e1^e6, e2^e8, e3^e7, e4^e8).  Linear in
// the bits of e, so swz(a | b) = swz(a) ^ swz(b) for disjoint bit sets.
__host__ __device__ __forceinline__ constexpr int swz(int e) {
    return e ^ (((e >> 5) & 1) | (((e >> 6) & 1) << 1) | (((e >> 8) & 1) << 2) |
                (((e >> 7) & 1) << 3) | (((e >> 8) & 1) << 4));
}

// --------------------------------------------------------- twiddle tables
// Per prime: 2048 pairs (w, floor(w * 2^32 / p)) with w canonical, for Shoup
// multiplication.  Entry m+i holds psi^brev11(m+i) (block i of the stage
// with m blocks) for m < 256; the last three stages (m = 256, 512, 1024;
// c = m/128 twiddles per thread) are restrided so that entry m + k*128 + t
// holds twiddle m + c*t + k.
struct TwiddleSet {
    uint2 t[2][D];   // [q1, q2]
};
constexpr int TW_WORDS = 4 * D;   // u32 words of a TwiddleSet in shared memory

// Table k (prime k) of a TwiddleSet copied to shared memory.
__device__ __forceinline__ const uint2 *tw_of(const uint32_t *smem_tw, int k) {
    return reinterpret_cast<const uint2 *>(smem_tw) + k * D;
}

// y * w mod p in [0, 2p) for any y < 2^32 (Shoup): wq = floor(w * 2^32 / p).
__device__ __forceinline__ uint32_t shoup_mul(uint32_t y, uint32_t w, uint32_t wq, uint32_t p) {
    const uint32_t q = __umulhi(y, wq);
    return y * w - q * p;
}

// -------------------------------------------------------- NTT butterflies
__device__ __forceinline__ void ct_bfly(uint32_t &x, uint32_t &y, uint2 w, uint32_t p) {
    uint32_t xr = min(x, x - 2 * p);
    uint32_t t = shoup_mul(y, w.x, w.y, p);
    x = xr + t;
    y = xr - t + 2 * p;
}

// Cooley-Tukey butterfly without reducing x: for x, y below B the outputs
// are below B + 2p (the Shoup product is below 2p for any 32-bit y).
__device__ __forceinline__ void ct_bfly_lazy(uint32_t &x, uint32_t &y, uint2 w, uint32_t p) {
    const uint32_t t = shoup_mul(y, w.x, w.y, p);
    const uint32_t xr = x;
    x = xr + t;
    y = xr - t + 2 * p;
}

// Gentleman-Sande butterfly with the twiddle -w: x + y and (x - y)(-w) =
// (y - x) w, both in [0, 2p) for inputs below 2p.
__device__ __forceinline__ void gs_bfly_neg(uint32_t &x, uint32_t &y, uint2 w, uint32_t p) {
    uint32_t s = x + y;
    uint32_t d = y - x + 2 * p;
    x = min(s, s - 2 * p);
    y = shoup_mul(d, w.x, w.y, p);
}

// Per-thread address bases of the three layouts (t: thread within group).
__device__ __forceinline__ int baseA(int t) { return swz(t); }
__device__ __forceinline__ int baseB(int t) { return swz(128 * (t >> 3) + (t & 7)); }
__device__ __forceinline__ int baseC(int t) { return swz(16 * t); }

// Forward NTT of one plane, layout A in, layout C out.  tw: forward table
// of this prime (shared memory).  buf: 2 x 2048 words of shared memory
// private to the group.  Value bounds (p < 2^28, 16p + 2^19 < 2^32 for
// both primes; a stage adds less than 2p to the bound of a lazy butterfly):
//   LAZY = 0  Harvey butterflies: in and out below 4p;
//   LAZY = 1  digit inputs below 2^19: lazy butterflies, one min(x, x - 8p)
//             before phase C; out below 2^19 + 14p;
//   LAZY = 2  inputs below 8p: as 1 with one more min(x, x - 8p) before
//             phase B; out below 14p.
// Lazy outputs are meant for Montgomery products, which take any 32-bit
// operand.
template <int LAZY = 0>
__device__ __forceinline__ void ntt_fwd(uint32_t (&v)[VPT], const uint2 *__restrict__ tw,
                                        uint32_t *buf, const Prime &c, int t, int bar_id) {
    const uint32_t p = c.p;
    // phase A: h = 1024, 512, 256, 128  (pairs j, j + 8>>L)
#pragma unroll
    for (int L = 0; L < 4; L++) {
        const int dj = 8 >> L;
#pragma unroll
        for (int j = 0; j < VPT; j++)
            if ((j & dj) == 0) {
                if constexpr (LAZY) ct_bfly_lazy(v[j], v[j + dj], tw[(1 << L) + j / (2 * dj)], p);
                else ct_bfly(v[j], v[j + dj], tw[(1 << L) + j / (2 * dj)], p);
            }
    }
    if constexpr (LAZY == 2) {
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = min(v[j], v[j] - 8 * p);
    }
    // transpose A -> B
    {
        uint32_t *b0 = buf;
        const int a = baseA(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) b0[a ^ swz(128 * j)] = v[j];
        group_sync(bar_id);
        const int b = baseB(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = b0[b ^ swz(8 * j)];
    }
    // phase B: h = 64, 32, 16, 8
    {
        const int bb = t >> 3;
#pragma unroll
        for (int L = 4; L < 8; L++) {
            const int dj = 8 >> (L - 4);
#pragma unroll
            for (int j = 0; j < VPT; j++)
                if ((j & dj) == 0) {
                    const uint2 w = tw[(1 << L) + (bb << (L - 4)) + (j >> (8 - L))];
                    if constexpr (LAZY) ct_bfly_lazy(v[j], v[j + dj], w, p);
                    else ct_bfly(v[j], v[j + dj], w, p);
                }
        }
    }
    if constexpr (LAZY) {
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = min(v[j], v[j] - 8 * p);
    }
    // transpose B -> C
    {
        uint32_t *b1 = buf + D;
        const int b = baseB(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) b1[b ^ swz(8 * j)] = v[j];
        group_sync(bar_id);
        const int cc = baseC(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = b1[cc ^ j];
    }
    // phase C: h = 4, 2, 1 (restrided twiddles)
#pragma unroll
    for (int L = 8; L < 11; L++) {
        const int dj = 4 >> (L - 8);
#pragma unroll
        for (int j = 0; j < VPT; j++)
            if ((j & dj) == 0) {
                if constexpr (LAZY) ct_bfly_lazy(v[j], v[j + dj], tw[(1 << L) + (j / (2 * dj)) * GROUP + t], p);
                else ct_bfly(v[j], v[j + dj], tw[(1 << L) + (j / (2 * dj)) * GROUP + t], p);
            }
    }
}

// Inverse NTT of one plane (without the 2048^-1 scaling).  v: layout C in
// (values < 2p), layout A out (values < 2p).  tw: this prime's FORWARD
// table: block i of the stage with m blocks uses -tw[2m-1-i] (in the
// restrided stages block c*t + k is entry m + (c-1-k)*128 + (127-t)).
__device__ __forceinline__ void ntt_inv(uint32_t (&v)[VPT], const uint2 *__restrict__ tw,
                                        uint32_t *buf, const Prime &c, int t, int bar_id) {
    const uint32_t p = c.p;
#pragma unroll
    for (int L = 10; L >= 8; L--) {
        const int dj = 4 >> (L - 8), cs = (1 << L) / GROUP;
#pragma unroll
        for (int j = 0; j < VPT; j++)
            if ((j & dj) == 0)
                gs_bfly_neg(v[j], v[j + dj], tw[(1 << L) + (cs - 1 - j / (2 * dj)) * GROUP + (GROUP - 1 - t)], p);
    }
    {
        uint32_t *b0 = buf;
        const int cc = baseC(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) b0[cc ^ j] = v[j];
        group_sync(bar_id);
        const int b = baseB(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = b0[b ^ swz(8 * j)];
    }
    {
        const int bb = t >> 3;
#pragma unroll
        for (int L = 7; L >= 4; L--) {
            const int dj = 8 >> (L - 4);
#pragma unroll
            for (int j = 0; j < VPT; j++)
                if ((j & dj) == 0)
                    gs_bfly_neg(v[j], v[j + dj], tw[(2 << L) - 1 - ((bb << (L - 4)) + (j >> (8 - L)))], p);
        }
    }
    {
        uint32_t *b1 = buf + D;
        const int b = baseB(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) b1[b ^ swz(8 * j)] = v[j];
        group_sync(bar_id);
        const int a = baseA(t);
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = b1[a ^ swz(128 * j)];
    }
#pragma unroll
    for (int L = 3; L >= 0; L--) {
        const int dj = 8 >> L;
#pragma unroll
        for (int j = 0; j < VPT; j++)
            if ((j & dj) == 0) gs_bfly_neg(v[j], v[j + dj], tw[(2 << L) - 1 - j / (2 * dj)], p);
    }
}

// Copy the two twiddle tables into shared memory (all threads of the CTA).
// Eight loads are issued before their stores, so a CTA pays about one L2
// latency per 8 x blockDim 16-byte words instead of one per word.
__device__ __forceinline__ void load_twiddles(uint32_t *dst, const TwiddleSet *src) {
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    constexpr int NW = TW_WORDS / 4;
    for (int i0 = threadIdx.x; i0 < NW; i0 += 8 * blockDim.x) {
        uint4 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int i = i0 + k * blockDim.x;
            if (i < NW) v[k] = __ldg(s + i);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int i = i0 + k * blockDim.x;
            if (i < NW) d[i] = v[k];
        }
    }
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialisation may start while its predecessor in the stream is still
// running; it must call pdl_wait() before it reads or writes anything the
// predecessor touches (the predecessor then has completed and its writes are
// visible).  pdl_launch_dependents() lets the next such kernel start early.
// Both are no-ops for a kernel launched the ordinary way.
// In an answer run the first expansion round is an ordinary launch, so it
// starts after the kernel that uploads the query descriptors has completed;
// every later kernel of the run starts after that round has, and may read
// its descriptor (for early exits) before its pdl_wait().
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Slot permutation of the automorphism x -> x^tau in NTT form: the slot z
// evaluates at psi^(2*brev(z)+1); tau(f) at that point is f at
// psi^((2*brev(z)+1)*tau), so out[z] = in[auto_slot(z, tau)].
__device__ __forceinline__ int auto_slot(int z, uint32_t tau) {
    uint32_t r = __brev((uint32_t)z) >> (32 - LOGD);
    uint32_t e = ((2 * r + 1) * tau) & (2 * D - 1);
    return (int)(__brev((e - 1) >> 1) >> (32 - LOGD));
}

__device__ __forceinline__ int bits_per(int t) { return (MOD_BITS + t - 1) / t; }

// 16 consecutive u32 (layout C slice) load/store helpers.
__device__ __forceinline__ void ld16(uint32_t (&v)[VPT], const uint32_t *p) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint4 x = q[i];
        v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
    }
}
// ld16 that reads through L2 only (data another CTA wrote in this launch)
__device__ __forceinline__ void ld16_l2(uint32_t (&v)[VPT], const uint32_t *p) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint4 x = __ldcg(q + i);
        v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
    }
}
__device__ __forceinline__ void st16(uint32_t *p, const uint32_t (&v)[VPT]) {
    uint4 *q = reinterpret_cast<uint4 *>(p);
#pragma unroll
    for (int i = 0; i < 4; i++) q[i] = make_uint4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}

}  // namespace sp
