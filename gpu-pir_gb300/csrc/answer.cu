// Query-dependent stages of the answer path: expansion, Regev->GSW
// conversion, folding, packing, modulus switching and serialisation.
//
// CTA shape everywhere: 256 threads = two NTT groups of 128; group g works
// modulo prime g.  Raw (56-bit) values are rebuilt by an inverse CRT of both
// groups' INTT outputs exchanged through shared memory.
#include <algorithm>
#include <cstdlib>
#include <string>
#include <utility>

#include "answer.cuh"

namespace sp {

namespace {

constexpr int THREADS = 256;
// shared memory: 2 twiddle tables + per group 2 transpose buffers
constexpr int SMEM_WORDS = TW_WORDS + 2 * 2 * D;
constexpr int SMEM_BYTES = SMEM_WORDS * 4;

struct Ctx {
    const uint32_t *tw;   // 2 tables (TW_WORDS words)
    uint32_t *buf;   // this group's two transpose buffers
    uint32_t *bufs;  // both groups' buffers (exchange area, 4*D words)
    Prime c;
    int g, t, bar;
};

__device__ __forceinline__ Ctx setup(uint32_t *smem, const TwiddleSet *tws) {
    load_twiddles(smem, tws);
    Ctx x;
    x.g = threadIdx.x >> 7;
    x.t = threadIdx.x & (GROUP - 1);
    x.c = prime_of(x.g);
    x.tw = smem;
    x.bufs = smem + TW_WORDS;
    x.buf = x.bufs + x.g * 2 * D;
    x.bar = 1 + x.g;
    __syncthreads();
    return x;
}

__device__ __forceinline__ const uint2 *tw_fwd(const Ctx &x) { return tw_of(x.tw, x.g); }
// the inverse transforms read the forward table too (common.cuh)
__device__ __forceinline__ const uint2 *tw_inv(const Ctx &x) { return tw_of(x.tw, x.g); }

// Both groups hold unscaled INTT outputs (layout A, < 2p) of the same
// polynomial mod their prime; returns the raw coefficients of this thread's
// layout-A positions (identical in both groups).  Uses the first buffer of
// each group as the exchange area; ends with a CTA barrier so the buffers
// are free again.
__device__ __forceinline__ void exchange_icrt(const Ctx &x, const uint32_t (&v)[VPT], uint64_t (&raw)[VPT]) {
    uint32_t *mine = x.bufs + x.g * 2 * D;
#pragma unroll
    for (int j = 0; j < VPT; j++) mine[x.t + GROUP * j] = v[j];
    __syncthreads();
    const uint32_t *a0 = x.bufs, *a1 = x.bufs + 2 * D;
#pragma unroll
    for (int j = 0; j < VPT; j++) {
        const int e = x.t + GROUP * j;
        raw[j] = icrt(a0[e], a1[e]);
    }
    __syncthreads();
}

// acc (layout C, < 2p) += ntt (< 4p) * key (Montgomery, canonical)
__device__ __forceinline__ void mac16(uint32_t (&acc)[VPT], const uint32_t (&v)[VPT], const uint32_t *key,
                                      const Prime &c) {
    uint32_t w[VPT];
    ld16(w, key);
#pragma unroll
    for (int j = 0; j < VPT; j++) acc[j] = reduce2(acc[j] + mont_mul(v[j], w[j], c.p, c.pinv), 2 * c.p);
}

// Digits (raw >> shift) & mask (mask below 2^32) from the two 32-bit halves.
__device__ __forceinline__ void digits(uint32_t (&d)[VPT], const uint64_t (&raw)[VPT], int shift, uint64_t mask) {
#pragma unroll
    for (int j = 0; j < VPT; j++) {
        const uint32_t lo = (uint32_t)raw[j], hi = (uint32_t)(raw[j] >> 32);
        d[j] = (shift < 32 ? __funnelshift_r(lo, hi, shift) : hi >> (shift - 32)) & (uint32_t)mask;
    }
}

__device__ __forceinline__ uint32_t to_mont(uint32_t x, const Prime &c) {  // canonical -> canonical Montgomery
    uint32_t y = mont_mul(x, c.r2, c.p, c.pinv);
    return min(y, y - c.p);
}


}  // namespace

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}

// ------------------------------------------------------------ conversions
__global__ void k_narrow(const uint64_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t total, int to_m) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const Prime c = prime_of((int)((i / D) & 1));
        // any u64 mod p: the high word first (32-bit), then one Montgomery
        // reduction of a value below p * 2^32
        const uint64_t v = in[i];
        const uint32_t x = mod_u64(((uint64_t)((uint32_t)(v >> 32) % c.p) << 32) | (uint32_t)v, c);
        out[i] = to_m ? to_mont(x, c) : x;
    }
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint64_t *__restrict__ out, uint64_t total, int from_m) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const Prime c = prime_of((int)((i / D) & 1));
        uint32_t x = in[i];
        if (from_m) {
            x = mont_mul(x, 1u, c.p, c.pinv);
            x = min(x, x - c.p);
        }
        out[i] = x;
    }
}

// Inputs of an answer run read straight from the lane's pinned staging (host
// memory the device addresses directly): block k copies descriptor k to the
// device and narrows query k (u64 [2 rows][2 primes][D]) into its slot's
// u32 planes, as k_narrow does.
// Block (b, k) of STAGE_BLOCKS per query: a thread issues its STAGE_VPT host
// loads together, then narrows them.
constexpr int STAGE_THREADS = 256, STAGE_VPT = 4, STAGE_BLOCKS = 4 * D / (STAGE_THREADS * STAGE_VPT);
__global__ void __launch_bounds__(STAGE_THREADS) k_stage_in(const QDesc *__restrict__ h_qd, QDesc *__restrict__ d_qd,
                                                            const uint64_t *__restrict__ h_query) {
    const int k = blockIdx.y;
    if (blockIdx.x == 0) {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(h_qd + k);
        uint32_t *dst = reinterpret_cast<uint32_t *>(d_qd + k);
        for (int w = threadIdx.x; w < (int)(sizeof(QDesc) / 4); w += blockDim.x) dst[w] = src[w];
    }
    uint32_t *q = const_cast<uint32_t *>(h_qd[k].query);
    const uint64_t *in = h_query + (size_t)k * 4 * D;
    const int i0 = blockIdx.x * STAGE_THREADS * STAGE_VPT + threadIdx.x;
    uint64_t v[STAGE_VPT];
#pragma unroll
    for (int u = 0; u < STAGE_VPT; u++) v[u] = in[i0 + u * STAGE_THREADS];
#pragma unroll
    for (int u = 0; u < STAGE_VPT; u++) {
        const int i = i0 + u * STAGE_THREADS;
        const Prime c = prime_of((i / D) & 1);
        q[i] = mod_u64(((uint64_t)((uint32_t)(v[u] >> 32) % c.p) << 32) | (uint32_t)v[u], c);
    }
}

cudaError_t launch_stage_in(const QDesc *h_qd, QDesc *d_qd, const uint64_t *h_query, int nq, cudaStream_t st) {
    static_assert(sizeof(QDesc) % 4 == 0, "descriptor words");
    static_assert(STAGE_BLOCKS * STAGE_THREADS * STAGE_VPT == 4 * D, "query tiling");
    k_stage_in<<<dim3(STAGE_BLOCKS, nq), STAGE_THREADS, 0, st>>>(h_qd, d_qd, h_query);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const uint64_t *in, uint32_t *out, uint64_t planes, bool to_mont, cudaStream_t st) {
    const uint64_t total = planes * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    if (blocks < 1) blocks = 1;
    k_narrow<<<blocks, 256, 0, st>>>(in, out, total, to_mont ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_widen(const uint32_t *in, uint64_t *out, uint64_t planes, bool from_mont, cudaStream_t st) {
    const uint64_t total = planes * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    if (blocks < 1) blocks = 1;
    k_widen<<<blocks, 256, 0, st>>>(in, out, total, from_mont ? 1 : 0);
    return cudaGetLastError();
}

// -------------------------------------------------------------- expansion
// Output i of round r (rows first..last of this group's prime g):
//   row 0 = v.row0 + acc0, row 1 = v.row1 + acc1 + tau(v.row1),
// v = ct (the parent) or, for an upper output, x^-(2^r) ct (n1 in NTT form).
// Written to the next round's buffer, to the GSW-bit inputs at the capture
// round and, for the last round's even outputs, staged in `bufs` and written
// as the first-dimension selector (one 16-byte slot [row 0 q1, row 0 q2,
// row 1 q1, row 1 q2] per coefficient).  Every thread of the CTA calls it.
__device__ __forceinline__ void expand_store(const QDesc &Q, int r, int i, bool upper, const uint32_t *ct,
                                             const uint32_t *n1, uint32_t tau, int max_bits, int first, int last,
                                             int g, int t, const Prime &c, uint32_t *bufs,
                                             const uint32_t (&acc0)[VPT], const uint32_t (&acc1)[VPT]) {
    const int zb = VPT * t;
    const bool to_sel = r == Q.g - 1 && !(i & 1) && (i / 2) < (1 << Q.nu1);
    if (to_sel) __syncthreads();   // every group is done with its transpose buffers
    for (int row = first; row <= last; row++) {
        const uint32_t *src = ct + (row * 2 + g) * D;
        uint32_t o[VPT];
        ld16(o, src + zb);
        if (upper) {
            uint32_t nn[VPT];
            ld16(nn, n1 + zb);
#pragma unroll
            for (int j = 0; j < VPT; j++) o[j] = reduce2(mont_mul(o[j], nn[j], c.p, c.pinv), c.p);
        }
#pragma unroll
        for (int j = 0; j < VPT; j++) o[j] = canon4(o[j] + (row == 0 ? acc0[j] : acc1[j]), c.p);
        if (row == 1) {
#pragma unroll
            for (int j = 0; j < VPT; j++) {
                const int zs = auto_slot(zb + j, tau);
                uint32_t tb = src[zs];
                if (upper) tb = reduce2(mont_mul(tb, n1[zs], c.p, c.pinv), c.p);
                o[j] = canon4(o[j] + tb, c.p);
            }
        }
        if (r + 1 < Q.g) st16(Q.v[(r + 1) & 1] + (size_t)i * 4 * D + (row * 2 + g) * D + zb, o);
        if (r == Q.capture && (i & 1) && (i / 2) < max_bits)
            st16(Q.gsw_in + (size_t)(i / 2) * 4 * D + (row * 2 + g) * D + zb, o);
        if (to_sel) st16(bufs + (row * 2 + g) * D + zb, o);
    }
    if (to_sel) {
        __syncthreads();
        uint4 *sl = reinterpret_cast<uint4 *>(Q.sel + (size_t)(i / 2) * D * 4);
        for (int z = threadIdx.x; z < D; z += blockDim.x)
            sl[z] = make_uint4(bufs[z], bufs[D + z], bufs[2 * D + z], bufs[3 * D + z]);
    }
}

// Round r for output index i = blockIdx.x of query blockIdx.y
// (gpu-pir/expansion.cuh:87-166 semantics): the input is v[i] for i < 2^r
// and x^(-2^r) * v[i - 2^r] above; the output is
//   v + [0; tau(v).row1] + W_r * NTT(G^-1(raw(tau(v).row0)))
// with tau = x -> x^(D/2^r + 1) applied as a slot permutation in NTT form.
// GP groups per prime split the t_exp digit transforms (GP = 2 for rounds
// with few outputs); with GP = 2 group (g, sub) finishes output row `sub`.
template <int GP>
__global__ void __launch_bounds__(256 * GP, 3 - GP) k_expand_round(const QDesc *__restrict__ qd, int r, StageParams sp,
                                                          const TwiddleSet *__restrict__ tws,
                                                          const uint32_t *__restrict__ neg1, int split,
                                                          uint32_t *__restrict__ part,
                                                          unsigned int *__restrict__ counters) {
    const QDesc &Q = qd[blockIdx.y];
    const int items = gridDim.x / split;
    const int i = blockIdx.x / split, s = blockIdx.x % split;
    __shared__ int s_last;
    if (!Q.active || r >= Q.g || i >= (2 << r)) return;
    const int max_bits = sp.t_gsw * Q.nu2;
    if (Q.stop > 0 && r > Q.stop && (i & 1)) return;
    if (Q.stop > 0 && r == Q.stop && (i & 1) && (i / 2) >= max_bits) return;
    extern __shared__ __align__(16) uint32_t smem[];
    pdl_launch_dependents();
    load_twiddles(smem, tws);   // constant: may overlap the previous round
    pdl_wait();
    const int gi = threadIdx.x >> 7, g = gi & 1, sub = gi >> 1, t = threadIdx.x & (GROUP - 1), bar = 1 + gi;
    const Prime c = prime_of(g);
    uint32_t *bufs = smem + TW_WORDS;
    uint32_t *buf = bufs + gi * 2 * D;
    const uint2 *twf = tw_of(smem, g), *twi = twf;
    __syncthreads();
    const int half = 1 << r;
    const bool upper = i >= half;
    const uint32_t *ct = r == 0 ? Q.query : Q.v[r & 1] + (size_t)(upper ? i - half : i) * 4 * D;
    const uint32_t *n1 = neg1 + ((size_t)r * 2 + g) * D;
    const uint32_t tau = (uint32_t)(D >> r) + 1;

    // raw(tau(row0)): INTT by the sub-0 group of each prime, inverse CRT by all
    if (sub == 0) {
        const uint32_t *row0 = ct + g * D;
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            const int zs = auto_slot(VPT * t + j, tau);
            const uint32_t a = row0[zs];
            v[j] = upper ? mont_mul(a, n1[zs], c.p, c.pinv) : a;   // (0, 2p)
        }
        ntt_inv(v, twi, buf, c, t, bar);
#pragma unroll
        for (int j = 0; j < VPT; j++) buf[t + GROUP * j] = v[j];   // first buffer free since the INTT's 2nd barrier
    }
    __syncthreads();
    // raw coefficients in shared memory (after the groups' buffers); each
    // group writes 16/(2*GP) of every thread's positions
    uint64_t *raws = reinterpret_cast<uint64_t *>(bufs + 2 * GP * 2 * D);
#pragma unroll
    for (int j = 0; j < VPT; j++) {
        if ((j * 2 * GP) / VPT != gi) continue;
        const int e = t + GROUP * j;
        raws[e] = icrt(bufs[e], bufs[2 * D + e]);
    }
    __syncthreads();
    const bool left = (r != 0) && !(i & 1);
    const int tk = left ? sp.t_left : sp.t_right;
    const uint32_t *W = (left ? Q.left : Q.right) + (size_t)r * 2 * tk * 2 * D;
    const int bits = bits_per(tk);
    const uint64_t mask = (1ull << bits) - 1;
    uint32_t acc0[VPT], acc1[VPT];
#pragma unroll
    for (int j = 0; j < VPT; j++) acc0[j] = acc1[j] = 0;
#pragma unroll 1
    for (int k = s * GP + sub; k < tk; k += GP * split) {
        uint32_t d[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            const uint2 x = reinterpret_cast<const uint2 *>(raws)[t + GROUP * j];
            const int sh = bits * k;
            d[j] = (sh < 32 ? __funnelshift_r(x.x, x.y, sh) : x.y >> (sh - 32)) & (uint32_t)mask;
        }
        ntt_fwd<1>(d, twf, buf, c, t, bar);   // digits below 2^19 (t >= 3)
        mac16(acc0, d, W + ((size_t)(0 * tk + k) * 2 + g) * D + VPT * t, c);
        mac16(acc1, d, W + ((size_t)(1 * tk + k) * 2 + g) * D + VPT * t, c);
    }
    if constexpr (GP == 2) {
        group_sync(bar);
        if (sub == 0) st16(buf + VPT * t, acc1); else st16(buf + VPT * t, acc0);
        __syncthreads();
        uint32_t w[VPT];
        ld16(w, bufs + (g + 2 * (1 - sub)) * 2 * D + VPT * t);
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            if (sub == 0) acc0[j] = reduce2(acc0[j] + w[j], 2 * c.p);
            else acc1[j] = reduce2(acc1[j] + w[j], 2 * c.p);
        }
        if (split > 1) {
            // publish this CTA's partial of row `sub`; the last CTA of the
            // output sums the others' and writes the output
            uint32_t(&a)[VPT] = sub == 0 ? acc0 : acc1;
            const size_t slot0 = ((size_t)blockIdx.y * items + i) * split;
            st16(part + ((slot0 + s) * 4 + g * 2 + sub) * D + VPT * t, a);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0)
                s_last = atomicAdd(&counters[(size_t)blockIdx.y * items + i], 1u) == (unsigned)(split - 1);
            __syncthreads();
            if (!s_last) return;
            __threadfence();
            for (int s2 = 0; s2 < split; s2++) {
                if (s2 == s) continue;
                ld16_l2(w, part + ((slot0 + s2) * 4 + g * 2 + sub) * D + VPT * t);
#pragma unroll
                for (int j = 0; j < VPT; j++) a[j] = reduce2(a[j] + w[j], 2 * c.p);
            }
            if (threadIdx.x == 0) counters[(size_t)blockIdx.y * items + i] = 0;   // ready for the next launch
        }
    }
    // GP = 2: group (g, sub) writes row `sub`
    expand_store(Q, r, i, upper, ct, n1, tau, max_bits, GP == 2 ? sub : 0, GP == 2 ? sub : 1, g, t, c, bufs, acc0,
                 acc1);
}

// Round r with many outputs: CTA blockIdx.x = parent p < 2^r of query
// blockIdx.y computes both children, p and p + 2^r (k_expand_round's
// outputs of those indices, the same residues).  With k = 2^r and
// tau = D / k + 1, tau(x^-k c) = -x^-k tau(c) (k * tau = D + k, x^D = -1),
// so the upper child's raw(tau(.).row0) is the lower's rotated by k with a
// sign change: one inverse transform and one gather per parent instead of
// two.  The children share the key (left for even indices, right for odd,
// and p + 2^r has p's parity for r >= 1; right for both at r = 0).
__global__ void __launch_bounds__(THREADS, 2) k_expand_pair(const QDesc *__restrict__ qd, int r, StageParams sp,
                                                           const TwiddleSet *__restrict__ tws,
                                                           const uint32_t *__restrict__ neg1) {
    const QDesc &Q = qd[blockIdx.y];
    const int pr = blockIdx.x, half = 1 << r;
    if (!Q.active || r >= Q.g || pr >= half) return;
    const int max_bits = sp.t_gsw * Q.nu2;
    auto live = [&](int i) {
        if (Q.stop > 0 && r > Q.stop && (i & 1)) return false;
        if (Q.stop > 0 && r == Q.stop && (i & 1) && (i / 2) >= max_bits) return false;
        return true;
    };
    const bool live_lo = live(pr), live_up = live(pr + half);
    if (!live_lo && !live_up) return;
    extern __shared__ __align__(16) uint32_t smem[];
    pdl_launch_dependents();
    load_twiddles(smem, tws);   // constant: may overlap the previous round
    pdl_wait();
    const int g = threadIdx.x >> 7, t = threadIdx.x & (GROUP - 1), bar = 1 + g;
    const Prime c = prime_of(g);
    uint32_t *bufs = smem + TW_WORDS;
    uint32_t *buf = bufs + g * 2 * D;
    const uint2 *twf = tw_of(smem, g), *twi = twf;
    __syncthreads();
    const uint32_t *ct = r == 0 ? Q.query : Q.v[r & 1] + (size_t)pr * 4 * D;
    const uint32_t *n1 = neg1 + ((size_t)r * 2 + g) * D;
    const uint32_t tau = (uint32_t)(D >> r) + 1;
    {
        // raw(tau(c.row0)) of the parent: INTT per prime, inverse CRT by all
        const uint32_t *row0 = ct + g * D;
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = row0[auto_slot(VPT * t + j, tau)];
        ntt_inv(v, twi, buf, c, t, bar);
#pragma unroll
        for (int j = 0; j < VPT; j++) buf[t + GROUP * j] = v[j];
    }
    __syncthreads();
    uint64_t *raws = reinterpret_cast<uint64_t *>(bufs + 2 * 2 * D);
#pragma unroll
    for (int j = 0; j < VPT; j++) {
        if ((j * 2) / VPT != g) continue;
        const int e = t + GROUP * j;
        raws[e] = icrt(bufs[e], bufs[2 * D + e]);
    }
    __syncthreads();
    const bool left = (r != 0) && !(pr & 1);
    const int tk = left ? sp.t_left : sp.t_right;
    const uint32_t *W = (left ? Q.left : Q.right) + (size_t)r * 2 * tk * 2 * D;
    const int bits = bits_per(tk);
    const uint32_t m32 = (uint32_t)((1ull << bits) - 1);
#pragma unroll 1
    for (int h = 0; h < 2; h++) {
        const int i = pr + h * half;
        const bool upper = h == 1;
        if (upper) {
            // raws <- -x^-k raws: position e takes -raws[e + k] below D - k,
            // raws[e + k - D] from there on (canonical mod q)
            uint64_t w[D / THREADS];
#pragma unroll
            for (int u = 0; u < D / THREADS; u++) {
                const int e = threadIdx.x + THREADS * u, src = e + half;
                if (src < D) {
                    const uint64_t a = raws[src];
                    w[u] = a ? QQ - a : 0;
                } else {
                    w[u] = raws[src - D];
                }
            }
            __syncthreads();   // every read of raws (and of the lower child's staging) done
#pragma unroll
            for (int u = 0; u < D / THREADS; u++) raws[threadIdx.x + THREADS * u] = w[u];
            __syncthreads();
        }
        if (!(upper ? live_up : live_lo)) continue;
        uint32_t acc0[VPT], acc1[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) acc0[j] = acc1[j] = 0;
#pragma unroll 1
        for (int k = 0; k < tk; k++) {
            uint32_t d[VPT];
            const int sh = bits * k;
#pragma unroll
            for (int j = 0; j < VPT; j++) {
                const uint2 x = reinterpret_cast<const uint2 *>(raws)[t + GROUP * j];
                d[j] = (sh < 32 ? __funnelshift_r(x.x, x.y, sh) : x.y >> (sh - 32)) & m32;
            }
            ntt_fwd<1>(d, twf, buf, c, t, bar);   // digits below 2^19 (t >= 3)
            mac16(acc0, d, W + ((size_t)(0 * tk + k) * 2 + g) * D + VPT * t, c);
            mac16(acc1, d, W + ((size_t)(1 * tk + k) * 2 + g) * D + VPT * t, c);
        }
        // v = c (lower child) or x^-k c (upper)
        expand_store(Q, r, i, upper, ct, n1, tau, max_bits, 0, 1, g, t, c, bufs, acc0, acc1);
    }
}

namespace {
// Expansion kernel of every round: chosen by size (launch_expand_round), or
// forced for all rounds by SPIRALPIR_EXPAND_KERNEL = split | single | pair,
// read once per process (the tests answer the same queries with each).
int expand_kernel_override() {
    static const int v = [] {
        const char *e = std::getenv("SPIRALPIR_EXPAND_KERNEL");
        if (!e) return 0;
        const std::string s(e);
        return s == "split" ? 1 : s == "single" ? 2 : s == "pair" ? 3 : 0;
    }();
    return v;
}
}  // namespace

cudaError_t launch_expand_round(const QDesc *qd, int nq, int r, int max_out, const StageParams &sp,
                                const TwiddleSet *tw, const uint32_t *neg1, const SplitScratch *scr,
                                cudaStream_t st, int split_shift) {
    // round 0 is an ordinary launch: the dependent launches after it read
    // their descriptors before their dependency wait (common.cuh)
    const uint64_t total = (uint64_t)max_out * nq;
    const int sms = sm_count();
    const int kernel = expand_kernel(max_out, nq, sms, expand_kernel_override());
    if (kernel == EXPAND_SPLIT) {
        // few outputs: 2 groups per prime split the digits; with scratch,
        // each output also spreads over `split` CTAs while that stays within
        // one CTA per SM, at least one digit transform per group
        int split = 1;
        if (scr && scr->part) {
            const int digits = std::max(sp.t_left, sp.t_right);
            split = shifted_split(split_rule(sms, total, (digits + 1) / 2), split_shift, (digits + 1) / 2);
            while (split > 1 && (total * split > (uint64_t)scr->slots || total > (uint64_t)scr->counter_slots)) split--;
        }
        const int smem = (TW_WORDS + 4 * 2 * D) * 4 + D * 8;
        cudaError_t e = cudaFuncSetAttribute(k_expand_round<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        e = launch_ex(k_expand_round<2>, dim3(max_out * split, nq), dim3(512), smem, st, r > 0, qd, r, sp, tw, neg1,
                      split, scr ? scr->part : nullptr, scr ? scr->counters : nullptr);
        if (e != cudaSuccess) return e;
    } else {
        const int smem = SMEM_BYTES + D * 8;
        cudaError_t e;
        if (kernel == EXPAND_PAIR) {
            // at least two waves of parents: one CTA per parent computes both
            // children (one inverse transform instead of two)
            e = cudaFuncSetAttribute(k_expand_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            e = launch_ex(k_expand_pair, dim3(std::max(1, max_out / 2), nq), dim3(THREADS), smem, st, r > 0, qd, r, sp,
                          tw, neg1);
        } else {
            // fewer: one CTA per output keeps every slot busy
            e = cudaFuncSetAttribute(k_expand_round<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            e = launch_ex(k_expand_round<1>, dim3(max_out, nq), dim3(THREADS), smem, st, r > 0, qd, r, sp, tw, neg1,
                          1, (uint32_t *)nullptr, (unsigned int *)nullptr);
        }
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// --------------------------------------------- DB-multiply output to raw
// Each CTA converts items blockIdx.x, blockIdx.x + gridDim.x, ... of its
// query (one polynomial = both primes' planes), so the twiddle tables are
// loaded once per CTA; the next item's planes are fetched while the current
// one is transformed.
__global__ void __launch_bounds__(THREADS, 2) k_acc_to_raw(const QDesc *__restrict__ qd, StageParams sp,
                                                          const TwiddleSet *__restrict__ tws) {
    pdl_launch_dependents();
    const QDesc &Q = qd[blockIdx.y];
    const int n_items = sp.T * (2 << Q.nu2);
    if (!Q.active || (int)blockIdx.x >= n_items) return;
    extern __shared__ __align__(16) uint32_t smem[];
    const Ctx x = setup(smem, tws);   // constant: may overlap the multiply's tail
    pdl_wait();                       // the multiply's accumulators
    uint32_t next[VPT];
    ld16(next, Q.acc + ((size_t)blockIdx.x * 2 + x.g) * D + VPT * x.t);
    for (int item = blockIdx.x; item < n_items; item += gridDim.x) {
        uint32_t v[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) v[j] = next[j];
        if (item + (int)gridDim.x < n_items)
            ld16(next, Q.acc + ((size_t)(item + gridDim.x) * 2 + x.g) * D + VPT * x.t);
        ntt_inv(v, tw_inv(x), x.buf, x.c, x.t, x.bar);
        uint64_t raw[VPT];
        exchange_icrt(x, v, raw);
        uint64_t *o = Q.raw + (size_t)item * D;
#pragma unroll
        for (int j = 0; j < VPT; j++)
            if ((j >> 3) == x.g) o[x.t + GROUP * j] = raw[j];
    }
}

cudaError_t launch_acc_to_raw(const QDesc *qd, int nq, int max_items, const StageParams &sp,
                              const TwiddleSet *tw, cudaStream_t st, bool pdl) {
    cudaError_t e = cudaFuncSetAttribute(k_acc_to_raw, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    // two resident CTAs per SM over all queries
    const int per_query = std::max(1, std::min(max_items, 2 * sm_count() / std::max(1, nq)));
    e = launch_ex(k_acc_to_raw, dim3(per_query, nq), dim3(THREADS), (size_t)SMEM_BYTES, st, pdl, qd, sp, tw);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

__global__ void k_sel_import(const uint64_t *__restrict__ in, uint32_t *__restrict__ sel, uint64_t total) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const int z = (int)(i % D);
        const uint64_t rk = i / D;            // row*4 + (ct_row*2 + prime)
        const int comp = (int)(rk % 4);
        const uint64_t row = rk / 4;
        sel[(row * D + z) * 4 + comp] = (uint32_t)in[i];
    }
}

cudaError_t launch_sel_import(const uint64_t *in, uint32_t *sel, int rows, cudaStream_t st) {
    const uint64_t total = (uint64_t)rows * 4 * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    k_sel_import<<<blocks, 256, 0, st>>>(in, sel, total);
    return cudaGetLastError();
}

// -------------------------------------------------------- Regev -> GSW
// Item blockIdx.x = dim*t_gsw + j: GSW column 2j+1 = the Regev encoding,
// column 2j = V * NTT(G^-1_{2,t_conv}(raw(c))).  Output in Montgomery form
// (the fold multiplies by it).
__global__ void __launch_bounds__(THREADS, 2) k_regev_to_gsw(const QDesc *__restrict__ qd, StageParams sp,
                                                         const TwiddleSet *__restrict__ tws) {
    const QDesc &Q = qd[blockIdx.y];
    const int idx = blockIdx.x;
    if (!Q.active || idx >= Q.nu2 * sp.t_gsw) return;
    extern __shared__ __align__(16) uint32_t smem[];
    const Ctx x = setup(smem, tws);
    const Prime &c = x.c;
    const int dim = idx / sp.t_gsw, jj = idx % sp.t_gsw;
    const int cols = 2 * sp.t_gsw;
    const uint32_t *ct = Q.gsw_in + (size_t)idx * 4 * D;
    uint32_t *G = Q.gsw + (size_t)dim * 2 * cols * 2 * D;
    const int bits = bits_per(sp.t_conv);
    const uint64_t mask = (1ull << bits) - 1;
    const int kc = 2 * sp.t_conv;
    uint32_t acc0[VPT], acc1[VPT];
#pragma unroll
    for (int j = 0; j < VPT; j++) acc0[j] = acc1[j] = 0;
#pragma unroll 1
    for (int row = 0; row < 2; row++) {
        uint64_t raw[VPT];
        {
            uint32_t v[VPT];
            ld16(v, ct + (row * 2 + x.g) * D + VPT * x.t);
            ntt_inv(v, tw_inv(x), x.buf, c, x.t, x.bar);
            exchange_icrt(x, v, raw);
        }
#pragma unroll 1
        for (int k = 0; k < sp.t_conv; k++) {
            uint32_t d[VPT];
            digits(d, raw, bits * k, mask);
            ntt_fwd<1>(d, tw_fwd(x), x.buf, c, x.t, x.bar);
            const int col = row + 2 * k;
            mac16(acc0, d, Q.conv + ((size_t)(0 * kc + col) * 2 + x.g) * D + VPT * x.t, c);
            mac16(acc1, d, Q.conv + ((size_t)(1 * kc + col) * 2 + x.g) * D + VPT * x.t, c);
        }
    }
    const int zb = VPT * x.t;
    uint32_t o[VPT];
#pragma unroll
    for (int j = 0; j < VPT; j++) o[j] = to_mont(reduce2(acc0[j], c.p), c);
    st16(G + ((size_t)(0 * cols + 2 * jj) * 2 + x.g) * D + zb, o);
#pragma unroll
    for (int j = 0; j < VPT; j++) o[j] = to_mont(reduce2(acc1[j], c.p), c);
    st16(G + ((size_t)(1 * cols + 2 * jj) * 2 + x.g) * D + zb, o);
    for (int row = 0; row < 2; row++) {
        ld16(o, ct + (row * 2 + x.g) * D + zb);
#pragma unroll
        for (int j = 0; j < VPT; j++) o[j] = to_mont(o[j], c);
        st16(G + ((size_t)(row * cols + 2 * jj + 1) * 2 + x.g) * D + zb, o);
    }
}

cudaError_t launch_regev_to_gsw(const QDesc *qd, int nq, int max_items, const StageParams &sp,
                                const TwiddleSet *tw, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(k_regev_to_gsw, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    k_regev_to_gsw<<<dim3(max_items, nq), THREADS, SMEM_BYTES, st>>>(qd, sp, tw);
    return cudaGetLastError();
}

// G - C (the NTT of the constant 2^(b k) is that constant in every slot).
__global__ void k_gsw_neg(const uint32_t *__restrict__ gsw, uint32_t *__restrict__ neg, uint64_t total, int t) {
    const int cols = 2 * t;
    const int bits = bits_per(t);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t r = i / D;
        const int k = (int)(r % 2); r /= 2;
        const int col = (int)(r % cols); r /= cols;
        const int row = (int)(r % 2);
        const Prime c = prime_of(k);
        uint32_t gval = 0;
        if ((col & 1) == row && bits * (col / 2) < 64) gval = (uint32_t)((1ull << (bits * (col / 2))) % c.p);
        uint32_t v = gval + c.p - gsw[i];
        neg[i] = v >= c.p ? v - c.p : v;
    }
}

cudaError_t launch_gsw_neg(const uint32_t *gsw, uint32_t *neg, int count, int t, cudaStream_t st) {
    const uint64_t total = (uint64_t)count * 2 * 2 * t * 2 * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 8192) blocks = 8192;
    k_gsw_neg<<<blocks, 256, 0, st>>>(gsw, neg, total, t);
    return cudaGetLastError();
}

// ----------------------------------------------------------------- fold
// Level `level`: v[i] <- v[i] + C * NTT(G^-1(v[num_per+i]) - G^-1(v[i])),
// which equals C*G^-1(v[num_per+i]) + (G - C)*G^-1(v[i]) exactly
// (G*G^-1(x) = x for the unsigned digits), the fold of
// gpu-pir/folding.cuh:9-27 with one product instead of two.
//
// GP groups of 128 threads per prime share one fold: the 2*t_gsw digit
// transforms are split between them, partial products are added through
// shared memory, and with GP = 2 each group finishes one output row.
// GP = 2 halves the latency of a fold and is used when a level has few folds.
template <int GP>
__global__ void __launch_bounds__(256 * GP, 3 - GP) k_fold_level(const QDesc *__restrict__ qd, int level, StageParams sp,
                                                        const TwiddleSet *__restrict__ tws, int split,
                                                        uint32_t *__restrict__ part,
                                                        unsigned int *__restrict__ counters) {
    const QDesc &Q = qd[blockIdx.y];
    if (!Q.active || level >= Q.nu2) return;
    const int items = gridDim.x / split;
    const int item = blockIdx.x / split, s = blockIdx.x % split;
    const int num_per = 1 << (Q.nu2 - 1 - level);
    const int inst = item / num_per, i = item % num_per;
    if (inst >= sp.T) return;
    __shared__ int s_last;
    extern __shared__ __align__(16) uint32_t smem[];
    pdl_launch_dependents();
    load_twiddles(smem, tws);   // constant: may overlap the previous level
    pdl_wait();
    const int gi = threadIdx.x >> 7, g = gi & 1, sub = gi >> 1, t = threadIdx.x & (GROUP - 1), bar = 1 + gi;
    const Prime c = prime_of(g);
    uint32_t *bufs = smem + TW_WORDS;           // [group][2][D]
    uint32_t *buf = bufs + gi * 2 * D;
    const uint2 *twf = tw_of(smem, g), *twi = twf;
    __syncthreads();
    const int cols = 1 << Q.nu2;
    uint64_t *base = Q.raw + (size_t)inst * cols * 2 * D;
    uint64_t *v0 = base + (size_t)i * 2 * D;
    const uint64_t *v1 = base + (size_t)(num_per + i) * 2 * D;
    const int tg = sp.t_gsw, gc = 2 * tg;
    const uint32_t *C = Q.gsw + (size_t)(Q.nu2 - 1 - level) * 2 * gc * 2 * D;
    const int bits = bits_per(tg);
    const uint64_t mask = (1ull << bits) - 1;
    uint32_t acc0[VPT], acc1[VPT];
#pragma unroll
    for (int j = 0; j < VPT; j++) acc0[j] = acc1[j] = 0;
#pragma unroll 1
    for (int pr = s * GP + sub; pr < 2 * tg; pr += GP * split) {
        const int row = pr / tg, k = pr % tg;
        const int sh = bits * k;
        // digit k of both inputs from 32-bit words: one word when the digit
        // lies in one half of the 64-bit value (fewer live registers), a
        // funnel shift of both halves when it straddles bit 32
        uint32_t d[VPT];
        const uint32_t m32 = (uint32_t)mask;
        const uint32_t *w1 = reinterpret_cast<const uint32_t *>(v1 + row * D);
        const uint32_t *w0 = reinterpret_cast<const uint32_t *>(v0 + row * D);
        if (sh + bits <= 32 || sh >= 32) {
            const int hw = sh >= 32, s2 = sh - 32 * hw;
#pragma unroll
            for (int j = 0; j < VPT; j++) {
                const int e = t + GROUP * j;
                const uint32_t a = (__ldg(w1 + 2 * e + hw) >> s2) & m32;
                const uint32_t b = (w0[2 * e + hw] >> s2) & m32;
                d[j] = a >= b ? a - b : a + c.p - b;
            }
        } else {
            const uint2 *u1 = reinterpret_cast<const uint2 *>(w1);
            const uint2 *u0 = reinterpret_cast<const uint2 *>(w0);
#pragma unroll
            for (int j = 0; j < VPT; j++) {
                const int e = t + GROUP * j;
                const uint2 x1 = __ldg(u1 + e), x0 = u0[e];
                const uint32_t a = __funnelshift_r(x1.x, x1.y, sh) & m32;
                const uint32_t b = __funnelshift_r(x0.x, x0.y, sh) & m32;
                d[j] = a >= b ? a - b : a + c.p - b;
            }
        }
        ntt_fwd<2>(d, twf, buf, c, t, bar);   // digit differences below p
        const int col = row + 2 * k;
        mac16(acc0, d, C + ((size_t)(0 * gc + col) * 2 + g) * D + VPT * t, c);
        mac16(acc1, d, C + ((size_t)(1 * gc + col) * 2 + g) * D + VPT * t, c);
    }
    if constexpr (GP == 1) {
        ntt_inv(acc0, twi, buf, c, t, bar);
        ntt_inv(acc1, twi, buf, c, t, bar);
        group_sync(bar);  // this group's last transpose reads are done
        uint32_t *ex0 = buf, *ex1 = buf + D;   // [prime][row] = bufs + (prime*2 + row)*D
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            ex0[t + GROUP * j] = acc0[j];
            ex1[t + GROUP * j] = acc1[j];
        }
        __syncthreads();
        const int row = g;   // group g finishes row g
        const uint32_t *a0 = bufs + row * D, *a1 = bufs + 2 * D + row * D;
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            const int e = t + GROUP * j;
            uint64_t y = icrt(a0[e], a1[e]) + v0[row * D + e];
            v0[row * D + e] = y >= QQ ? y - QQ : y;
        }
    } else {
        // group (g, sub) finishes row `sub`: hand the other row to the partner
        group_sync(bar);
        if (sub == 0) st16(buf + VPT * t, acc1); else st16(buf + VPT * t, acc0);
        __syncthreads();
        uint32_t w[VPT];
        ld16(w, bufs + (g + 2 * (1 - sub)) * 2 * D + VPT * t);
        uint32_t a[VPT];
#pragma unroll
        for (int j = 0; j < VPT; j++) a[j] = reduce2((sub == 0 ? acc0[j] : acc1[j]) + w[j], 2 * c.p);
        __syncthreads();   // partner has read this group's buffer
        if (split > 1) {
            // publish this CTA's partial; the last CTA of the item finishes it
            const size_t slot0 = ((size_t)blockIdx.y * items + item) * split;
            st16(part + ((slot0 + s) * 4 + g * 2 + sub) * D + VPT * t, a);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0)
                s_last = atomicAdd(&counters[(size_t)blockIdx.y * items + item], 1u) == (unsigned)(split - 1);
            __syncthreads();
            if (!s_last) return;
            __threadfence();
            for (int s2 = 0; s2 < split; s2++) {
                if (s2 == s) continue;
                ld16_l2(w, part + ((slot0 + s2) * 4 + g * 2 + sub) * D + VPT * t);
#pragma unroll
                for (int j = 0; j < VPT; j++) a[j] = reduce2(a[j] + w[j], 2 * c.p);
            }
            if (threadIdx.x == 0) counters[(size_t)blockIdx.y * items + item] = 0;   // ready for the next launch
        }
        ntt_inv(a, twi, buf, c, t, bar);
        group_sync(bar);
#pragma unroll
        for (int j = 0; j < VPT; j++) buf[t + GROUP * j] = a[j];
        __syncthreads();
        const int row = sub;
        const uint32_t *a0 = bufs + (2 * row) * 2 * D, *a1 = bufs + (1 + 2 * row) * 2 * D;
#pragma unroll
        for (int j = 0; j < VPT; j++) {
            if ((j >> 3) != g) continue;     // the two primes' groups split the positions
            const int e = t + GROUP * j;
            uint64_t y = icrt(a0[e], a1[e]) + v0[row * D + e];
            v0[row * D + e] = y >= QQ ? y - QQ : y;
        }
    }
}

cudaError_t launch_fold_level(const QDesc *qd, int nq, int level, int max_items, const StageParams &sp,
                              const TwiddleSet *tw, const SplitScratch *scr, cudaStream_t st, int split_shift,
                              bool pdl_first) {
    const bool pdl = level > 0 || pdl_first;
    const uint64_t total = (uint64_t)max_items * nq;
    const int sms = sm_count();
    if (fold_narrow(total, sms)) {
        // few folds (one CTA per SM): 2 groups per prime split the digits;
        // above that one 256-thread CTA per fold, two per SM, finishes a
        // level in one wave up to 2 x SMs folds.  With scratch, each
        // fold also spreads over `split` CTAs while that stays within one CTA
        // per SM (this kernel's footprint), at least one digit transform per
        // group
        int split = 1;
        if (scr && scr->part) {
            split = shifted_split(split_rule(sms, total, sp.t_gsw), split_shift, sp.t_gsw);
            while (split > 1 && (total * split > (uint64_t)scr->slots || total > (uint64_t)scr->counter_slots)) split--;
        }
        const int smem = (TW_WORDS + 4 * 2 * D) * 4;
        cudaError_t e = cudaFuncSetAttribute(k_fold_level<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        e = launch_ex(k_fold_level<2>, dim3(max_items * split, nq), dim3(512), smem, st, pdl, qd, level, sp, tw,
                      split, scr ? scr->part : nullptr, scr ? scr->counters : nullptr);
        if (e != cudaSuccess) return e;
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_fold_level<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        e = launch_ex(k_fold_level<1>, dim3(max_items, nq), dim3(THREADS), (size_t)SMEM_BYTES, st, pdl, qd, level,
                      sp, tw, 1, (uint32_t *)nullptr, (unsigned int *)nullptr);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// ----------------------------------------------------------------- pack
// floor(2^96 / q): floor(2^(64+b) / q) = RESCALE_M32 >> (32 - b) for b <= 32
constexpr uint64_t RESCALE_M32 = 0x1136db7cb1full;
static_assert(RESCALE_M32 == (uint64_t)(((unsigned __int128)1 << 96) / QQ), "reciprocal of q");

__device__ __forceinline__ uint32_t rescale_q(uint64_t x, int bits_out) {
    // round(x * 2^bits_out / q) mod 2^bits_out (bits_out <= 32), x read as
    // centred in Z_q: y = floor((a * 2^bits_out + floor(q/2)) / q).  Integer
    // only (GB300's FP64 rate is a small fraction of its integer rate): the
    // fixed-point reciprocal gives y or y - 1 or y - 2 (its error times a is
    // below 2^-8), and the remainder, below 3q < 2^58, is exact in wrapping
    // 64-bit arithmetic.
    const uint64_t mask = bits_out == 32 ? 0xffffffffull : (1ull << bits_out) - 1;
    const bool neg = x >= (QQ + 1) / 2;
    const uint64_t a = neg ? QQ - x : x;
    uint64_t y = __umul64hi(a, RESCALE_M32 >> (32 - bits_out));
    const uint64_t rem = (a << bits_out) + QQ / 2 - y * QQ;
    y += (rem >= QQ) + (rem >= 2 * QQ);
    y &= mask;
    return (uint32_t)(neg ? ((0 - y) & mask) : y);
}

// The response: n*D values of q2_bits (row 0 of each column), then n*n*D
// values of pt_bits + 2 (rows 1..n, row-major), least significant bit first
// in little-endian 32-bit words.  A polynomial holds D * b = 64 * b words,
// so each starts on a word boundary: first word of row a, column col.
__device__ __forceinline__ uint32_t *poly_words(const QDesc &Q, const StageParams &sp, int a, int col) {
    const size_t w0 = (size_t)(D / 32) * sp.q2_bits, w1 = (size_t)(D / 32) * (sp.pt_bits + 2);
    const size_t w = a == 0 ? col * w0 : sp.n * w0 + (size_t)((a - 1) * sp.n + col) * w1;
    return reinterpret_cast<uint32_t *>(Q.resp) + w;
}

// Raw coefficients of one response polynomial (this thread's layout-A
// positions, the same in both groups) -> rescaled to b bits and serialised
// into its 64 * b words at `out`.  Uses group 0's first transpose buffer;
// ends with a CTA barrier.
__device__ __forceinline__ void store_poly_bits(const Ctx &x, const uint64_t (&raw)[VPT], int b, uint32_t *out) {
    uint32_t *vals = x.bufs;
    if (x.g == 0) {
#pragma unroll
        for (int j = 0; j < VPT; j++) vals[x.t + GROUP * j] = rescale_q(raw[j], b);
    }
    __syncthreads();
    const int words = (D / 32) * b;
    for (int w = threadIdx.x; w < words; w += blockDim.x) {
        const int lo = w * 32;
        uint64_t acc = 0;
        for (int e = lo / b; e < D && e * b < lo + 32; e++) {
            const int off = e * b - lo;
            const uint64_t v = vals[e];
            acc |= off >= 0 ? (v << off) : (v >> -off);
        }
        out[w] = (uint32_t)acc;
    }
    __syncthreads();
}

// Column col of query blockIdx.y: sum over r < n of
// W_r * NTT(G^-1(ct[r*n+col].row0)) + e_{1+r} * NTT(ct[r*n+col].row1), then
// raw, then row 0 rescaled to 2^q2_bits and rows 1..n to 4p, serialised into
// the response.
// The n*(t_conv + 1) transforms of a column (digit k < t_conv of ct r's row
// 0, or its row 1 for k = t_conv) are spread over `split` CTAs; with
// split > 1 each CTA publishes its partial sums and the last to arrive
// finishes the column (no CTA waits for another).  PACK_MAX_N (2 or 4) bounds
// n: the n + 1 accumulators live in registers.  The last kernel of a run
// (in stream order, or dependent on the last fold level): after the wait,
// block (0, 0) passes the run's error flag to h_err when given.
template <int PACK_MAX_N>
__global__ void __launch_bounds__(THREADS, PACK_MAX_N <= 2 ? 2 : 1) k_pack(const QDesc *__restrict__ qd, StageParams sp,
                                                 const TwiddleSet *__restrict__ tws, int split,
                                                 uint32_t *__restrict__ part, unsigned int *__restrict__ counters,
                                                 const int *__restrict__ d_err, int *__restrict__ h_err) {
    pdl_wait();
    if (h_err && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *h_err = *d_err;
    const QDesc &Q = qd[blockIdx.y];
    const int col = blockIdx.x / split, s = blockIdx.x % split;
    if (!Q.active || col >= sp.n) return;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ int s_last;
    const Ctx x = setup(smem, tws);
    const Prime &c = x.c;
    const int n = sp.n, tcv = sp.t_conv;
    const int cols = 1 << Q.nu2;
    const int bits = bits_per(tcv);
    const uint64_t mask = (1ull << bits) - 1;
    uint32_t acc[PACK_MAX_N + 1][VPT];
#pragma unroll
    for (int a = 0; a <= PACK_MAX_N; a++)
#pragma unroll
        for (int j = 0; j < VPT; j++) acc[a][j] = 0;
#pragma unroll 1
    for (int u = s; u < n * (tcv + 1); u += split) {
        const int r = u / (tcv + 1), k = u % (tcv + 1);
        const uint64_t *ct = Q.raw + (size_t)(r * n + col) * cols * 2 * D;   // folded result of instance r*n+col
        if (k < tcv) {
            const uint32_t *W = Q.pack + (size_t)r * (n + 1) * tcv * 2 * D;
            uint64_t raw[VPT];
#pragma unroll
            for (int j = 0; j < VPT; j++) raw[j] = ct[x.t + GROUP * j];
            uint32_t d[VPT];
            digits(d, raw, bits * k, mask);
            ntt_fwd<1>(d, tw_fwd(x), x.buf, c, x.t, x.bar);
#pragma unroll
            for (int a = 0; a <= PACK_MAX_N; a++)
                if (a <= n) mac16(acc[a], d, W + ((size_t)(a * tcv + k) * 2 + x.g) * D + VPT * x.t, c);
        } else {
            uint32_t b[VPT];
#pragma unroll
            for (int j = 0; j < VPT; j++) b[j] = mod_u64(ct[D + x.t + GROUP * j], c);
            ntt_fwd(b, tw_fwd(x), x.buf, c, x.t, x.bar);
#pragma unroll
            for (int j = 0; j < VPT; j++) b[j] = reduce2(b[j], 2 * c.p);
#pragma unroll
            for (int a = 1; a <= PACK_MAX_N; a++) {
                // row 1 of ct r goes to acc[1 + r]: a select, not an index
                // (an index would move acc to local memory)
                const uint32_t on = (a == 1 + r) ? 0xffffffffu : 0u;
#pragma unroll
                for (int j = 0; j < VPT; j++) acc[a][j] = reduce2(acc[a][j] + (b[j] & on), 2 * c.p);
            }
        }
    }
    if (split > 1) {
        const size_t item = (size_t)blockIdx.y * n + col;
        auto plane = [&](int s2, int a) { return part + (((item * split + s2) * (n + 1) + a) * 2 + x.g) * D + VPT * x.t; };
#pragma unroll
        for (int a = 0; a <= PACK_MAX_N; a++)
            if (a <= n) st16(plane(s, a), acc[a]);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(&counters[item], 1u) == (unsigned)(split - 1);
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        for (int s2 = 0; s2 < split; s2++) {
            if (s2 == s) continue;
#pragma unroll
            for (int a = 0; a <= PACK_MAX_N; a++) {
                if (a <= n) {
                    uint32_t w[VPT];
                    ld16_l2(w, plane(s2, a));
#pragma unroll
                    for (int j = 0; j < VPT; j++) acc[a][j] = reduce2(acc[a][j] + w[j], 2 * c.p);
                }
            }
        }
        if (threadIdx.x == 0) counters[item] = 0;   // ready for the next launch
    }
#pragma unroll
    for (int a = 0; a <= PACK_MAX_N; a++) {
        if (a > n) break;
        ntt_inv(acc[a], tw_inv(x), x.buf, c, x.t, x.bar);
        uint64_t raw[VPT];
        exchange_icrt(x, acc[a], raw);
        store_poly_bits(x, raw, a == 0 ? sp.q2_bits : sp.pt_bits + 2, poly_words(Q, sp, a, col));
    }
}

// The pack when every response polynomial of the launch can have its own
// SM: CTA blockIdx.x = item * split + s of query blockIdx.y computes only
// row a of column col (item = a * n + col): the key products
// W_r[a] * NTT(digit k of ct[r*n+col].row0) for r < n, k < t_conv, and for
// a >= 1 the row 1 of ct[(a-1)*n+col] (the e_{1+r} term of k_pack).  Those
// units are spread over `split` CTAs; the last to arrive sums the partials
// and finishes the polynomial, so the n + 1 rows of a column finish on
// different SMs at once instead of one after another.  One accumulator:
// any n.  The last kernel of a run: the twiddle load may overlap the last
// fold level; after the wait, block (0, 0) passes the error flag.
__global__ void __launch_bounds__(THREADS, 2) k_pack_row(const QDesc *__restrict__ qd, StageParams sp,
                                                        const TwiddleSet *__restrict__ tws, int split,
                                                        uint32_t *__restrict__ part,
                                                        unsigned int *__restrict__ counters,
                                                        const int *__restrict__ d_err, int *__restrict__ h_err) {
    const QDesc &Q = qd[blockIdx.y];
    const int n = sp.n, tcv = sp.t_conv, items = n * (n + 1);
    const int item = blockIdx.x / split, s = blockIdx.x % split;
    const int a = item / n, col = item % n;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ int s_last;
    const Ctx x = setup(smem, tws);   // twiddles: constant, may overlap the last fold level
    pdl_wait();
    if (h_err && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *h_err = *d_err;
    if (!Q.active || item >= items) return;
    const Prime &c = x.c;
    const int cols = 1 << Q.nu2;
    const int bits = bits_per(tcv);
    const uint64_t mask = (1ull << bits) - 1;
    const int units = n * tcv + (a > 0);
    uint32_t acc[VPT];
#pragma unroll
    for (int j = 0; j < VPT; j++) acc[j] = 0;
#pragma unroll 1
    for (int u = s; u < units; u += split) {
        if (u < n * tcv) {
            const int r = u / tcv, k = u % tcv;
            const uint64_t *ct = Q.raw + (size_t)(r * n + col) * cols * 2 * D;
            const uint32_t *W = Q.pack + (size_t)r * (n + 1) * tcv * 2 * D;
            uint64_t raw[VPT];
#pragma unroll
            for (int j = 0; j < VPT; j++) raw[j] = ct[x.t + GROUP * j];
            uint32_t d[VPT];
            digits(d, raw, bits * k, mask);
            ntt_fwd<1>(d, tw_fwd(x), x.buf, c, x.t, x.bar);
            mac16(acc, d, W + ((size_t)(a * tcv + k) * 2 + x.g) * D + VPT * x.t, c);
        } else {
            const uint64_t *ct = Q.raw + (size_t)((a - 1) * n + col) * cols * 2 * D;
            uint32_t b[VPT];
#pragma unroll
            for (int j = 0; j < VPT; j++) b[j] = mod_u64(ct[D + x.t + GROUP * j], c);
            ntt_fwd(b, tw_fwd(x), x.buf, c, x.t, x.bar);
#pragma unroll
            for (int j = 0; j < VPT; j++) acc[j] = reduce2(acc[j] + reduce2(b[j], 2 * c.p), 2 * c.p);
        }
    }
    if (split > 1) {
        const size_t slot = (size_t)blockIdx.y * items + item;
        auto plane = [&](int s2) { return part + ((slot * split + s2) * 2 + x.g) * D + VPT * x.t; };
        st16(plane(s), acc);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(&counters[slot], 1u) == (unsigned)(split - 1);
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        for (int s2 = 0; s2 < split; s2++) {
            if (s2 == s) continue;
            uint32_t w[VPT];
            ld16_l2(w, plane(s2));
#pragma unroll
            for (int j = 0; j < VPT; j++) acc[j] = reduce2(acc[j] + w[j], 2 * c.p);
        }
        if (threadIdx.x == 0) counters[slot] = 0;   // ready for the next launch
    }
    ntt_inv(acc, tw_inv(x), x.buf, c, x.t, x.bar);
    uint64_t raw[VPT];
    exchange_icrt(x, acc, raw);
    store_poly_bits(x, raw, a == 0 ? sp.q2_bits : sp.pt_bits + 2, poly_words(Q, sp, a, col));
}

cudaError_t launch_pack(const QDesc *qd, int nq, const StageParams &sp, const TwiddleSet *tw,
                        const SplitScratch *scr, cudaStream_t st, int split_shift, const int *d_err, int *h_err,
                        bool pdl) {
    const int sms = sm_count();
    if (pack_by_row(sp.n, nq, sms, scr && scr->part, scr ? scr->counter_slots : 0)) {
        // one SM per response polynomial: spread each one's key products
        const uint64_t items = (uint64_t)sp.n * (sp.n + 1) * nq;
        const int units = sp.n * sp.t_conv + 1;
        int split = shifted_split(split_rule(sms, items, units), split_shift, units);
        while (split > 1 && items * split * 2 > (uint64_t)scr->slots * 4) split--;
        cudaError_t e = cudaFuncSetAttribute(k_pack_row, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        if (e != cudaSuccess) return e;
        e = launch_ex(k_pack_row, dim3(sp.n * (sp.n + 1) * split, nq), dim3(THREADS), (size_t)SMEM_BYTES, st, pdl, qd,
                      sp, tw, split, scr->part, scr->counters, d_err, h_err);
        if (e != cudaSuccess) return e;
        return cudaGetLastError();
    }
    auto kernel = sp.n <= 2 ? k_pack<2> : k_pack<4>;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    // spread each column's n*(t_conv+1) transforms over CTAs while the launch
    // stays within the SMs and the scratch
    const uint64_t cols = (uint64_t)sp.n * nq;
    const int units = sp.n * (sp.t_conv + 1);
    int split = 1;
    if (scr && scr->part) {
        split = shifted_split(split_rule(sms, cols, units), split_shift, units);
        while (split > 1 && (cols * split * (sp.n + 1) * 2 > (uint64_t)scr->slots * 4 || cols > (uint64_t)scr->counter_slots))
            split--;
    }
    e = launch_ex(kernel, dim3(sp.n * split, nq), dim3(THREADS), (size_t)SMEM_BYTES, st, pdl, qd, sp, tw, split,
                  scr ? scr->part : nullptr, scr ? scr->counters : nullptr, d_err, h_err);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

uint64_t response_bytes(const StageParams &sp) {
    const uint64_t bits = (uint64_t)sp.n * D * sp.q2_bits + (uint64_t)sp.n * sp.n * D * (sp.pt_bits + 2);
    return (bits + 63) / 64 * 8;
}

}  // namespace sp
