// Per-query descriptors and launchers of the query-dependent stages:
// coefficient expansion (R6, R7, R8), Regev->GSW conversion (R9), G - C
// (R10), DB-multiply output to raw (R13), folding (R12) and packing /
// modulus switching / serialisation (R14).
//
// Every kernel takes an array of QDesc (one per query of the launch) so that
// queries against databases of different shapes run in the same launch.
#pragma once
#include "kernels.cuh"
#include "plan.h"

namespace sp {

// Scratch of split launches: a narrow fold level (or expansion round) may
// run each item as `split` CTAs that transform disjoint subsets of the
// digits; each CTA stores its partial key products and the last to arrive
// (arrival counter per item, no waiting) sums them and finishes the item.
struct SplitScratch {
    uint32_t *part = nullptr;       // [slots][2 primes x 2 rows][D] partial sums
    uint32_t *counters = nullptr;   // [counter_slots], zero between launches
    int slots = 0, counter_slots = 0;
};

// u64 canonical residues [count][2][D] -> u32 (optionally Montgomery form)
cudaError_t launch_narrow(const uint64_t *in, uint32_t *out, uint64_t planes, bool to_mont, cudaStream_t st);
// u32 [count][2][D] (optionally from Montgomery form) -> u64 canonical
cudaError_t launch_widen(const uint32_t *in, uint64_t *out, uint64_t planes, bool from_mont, cudaStream_t st);

// The `pdl` flags below launch a kernel dependent on the previous kernel of
// the stream (programmatic dependent launch): it starts as that one's CTAs
// retire and waits for it to complete before reading its outputs.

// DB-multiply output (NTT form) -> raw fold input, every query of qd
cudaError_t launch_acc_to_raw(const QDesc *qd, int nq, int max_items, const StageParams &sp,
                              const TwiddleSet *tw, cudaStream_t st, bool pdl = false);
// selectors u64 [rows][2 rows][2][D] -> device selector layout u32 [rows][D][4]
cudaError_t launch_sel_import(const uint64_t *in, uint32_t *sel, int rows, cudaStream_t st);

cudaError_t launch_expand_round(const QDesc *qd, int nq, int r, int max_out, const StageParams &sp,
                                const TwiddleSet *tw, const uint32_t *neg1, const SplitScratch *scr,
                                cudaStream_t st, int split_shift = 0);
cudaError_t launch_regev_to_gsw(const QDesc *qd, int nq, int max_items, const StageParams &sp,
                                const TwiddleSet *tw, cudaStream_t st);
// G - C for count GSW ciphertexts (canonical in and out)
cudaError_t launch_gsw_neg(const uint32_t *gsw, uint32_t *neg, int count, int t, cudaStream_t st);
// scr == nullptr: no split (every item in one CTA).  Levels after the first
// are dependent launches; the first one too with pdl_first.
cudaError_t launch_fold_level(const QDesc *qd, int nq, int level, int max_items, const StageParams &sp,
                              const TwiddleSet *tw, const SplitScratch *scr, cudaStream_t st, int split_shift = 0,
                              bool pdl_first = false);
// Pack, modulus switch and serialise each query's response to Q.resp (device
// memory, or pinned host memory for runs with host I/O): one launch, after
// every other kernel of the run; with h_err, it also copies *d_err to *h_err.
cudaError_t launch_pack(const QDesc *qd, int nq, const StageParams &sp, const TwiddleSet *tw,
                        const SplitScratch *scr, cudaStream_t st, int split_shift = 0, const int *d_err = nullptr,
                        int *h_err = nullptr, bool pdl = false);
// Descriptors h_qd[0, nq) (pinned host memory) to d_qd, and the u64 queries
// h_query[nq][2][2][D] (pinned) narrowed into each descriptor's query planes.
cudaError_t launch_stage_in(const QDesc *h_qd, QDesc *d_qd, const uint64_t *h_query, int nq, cudaStream_t st);

uint64_t response_bytes(const StageParams &sp);

}  // namespace sp
