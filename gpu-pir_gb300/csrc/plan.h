// Launch and batching rules of the answer path as plain host functions (no
// CUDA): which kernel runs an expansion round, how a narrow launch spreads
// its items over CTAs, which pack kernel runs, and which queued requests the
// serving loop's next batch takes.  The launchers (answer.cu) and the
// serving loop (api.cu) call these; tests/test_plan_rules.py compiles this
// header on the CPU and checks the rules.
#pragma once
#include <stdint.h>

namespace sp {

// Split schedules of the narrow launches (few items: an expansion round, a
// fold level or the pack spreads each item over `split` CTAs).  The rule
// gives split = min(SMs / items, cap), at least 1; a schedule shifts it:
// shift s >= 0 multiplies it by 2^s, s < 0 divides it by 2^-s, SPLIT_NONE
// runs one CTA per item; the result stays in [1, cap].  Chosen per batch
// class by the autotuner (api.cu); every schedule gives the same residues.
constexpr int SPLIT_NONE = -16;
inline int split_rule(uint64_t sms, uint64_t items, uint64_t cap) {
    uint64_t r = items ? sms / items : sms;
    if (r < 1) r = 1;
    return (int)(r < cap ? r : cap);
}
inline int shifted_split(int rule, int shift, int cap) {
    if (shift <= SPLIT_NONE) return 1;
    const int s = shift >= 0 ? rule << shift : rule >> -shift;
    return s < 1 ? 1 : (s > cap ? cap : s);
}

// Kernel of an expansion round with max_out outputs per query (2^(r+1)
// before pruning) for nq queries:
//  - EXPAND_SPLIT (k_expand_round<2>): fewer outputs than two per SM; two
//    groups per prime split the digits and each output spreads over CTAs;
//  - EXPAND_PAIR (k_expand_pair): at least two waves of parents (4 per SM);
//    one CTA computes both children of a parent from one inverse transform;
//  - EXPAND_SINGLE (k_expand_round<1>): one CTA per output otherwise.
// force (1, 2 or 3) runs that kernel for every round.
enum ExpandKernel { EXPAND_SPLIT = 1, EXPAND_SINGLE = 2, EXPAND_PAIR = 3 };
inline int expand_kernel(uint64_t max_out, uint64_t nq, uint64_t sms, int force) {
    if (force >= EXPAND_SPLIT && force <= EXPAND_PAIR) return force;
    if (max_out * nq < 2 * sms) return EXPAND_SPLIT;
    const uint64_t pairs = (max_out / 2 > 1 ? max_out / 2 : 1) * nq;
    return pairs >= 4 * sms ? EXPAND_PAIR : EXPAND_SINGLE;
}

// A fold level of `folds` folds over all queries runs 512-thread CTAs that
// split the digit transforms (k_fold_level<2>) when it has at most one fold
// per SM, else one 256-thread CTA per fold, two per SM (k_fold_level<1>).
inline bool fold_narrow(uint64_t folds, uint64_t sms) { return folds <= sms; }

// The pack gives each output polynomial (row a, column) its own CTAs
// (k_pack_row) when all n (n + 1) of them over nq queries fit one per SM and
// the split scratch is there; else one CTA group per column (k_pack).
inline bool pack_by_row(int n, uint64_t nq, uint64_t sms, bool scratch, uint64_t counter_slots) {
    const uint64_t items = (uint64_t)n * (n + 1) * nq;
    return scratch && items <= sms && items <= counter_slots;
}

// The serving loop's next batch on a lane with `cap` slots while `queued`
// requests wait, oldest first.  A queue that fits in one batch runs whole,
// in arrival order.  A longer one runs by database: the oldest request's
// database first, with its other queued requests (up to the capacity, in
// arrival order), so that one pass over a database image serves as many
// queries as wait for it; requests for other databases keep their place.
struct BatchRule {
    bool by_db;
    int db;
    bool takes(int db_id) const { return !by_db || db_id == db; }
};
inline BatchRule batch_rule(uint64_t queued, int cap, int oldest_db) {
    return BatchRule{queued > (uint64_t)cap, oldest_db};
}

}  // namespace sp
