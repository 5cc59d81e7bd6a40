// C ABI of the Spiral answer path (include/spiralpir.h): context, device
// memory under an HBM budget, databases, client keys, the answer pipeline
// and the stage entry points used by the parity tests.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <condition_variable>
#include <deque>
#include <chrono>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/spiralpir.h"
#include "answer.cuh"
#include "ctx_view.h"
#include "seeded.cuh"

using namespace sp;

namespace {

thread_local std::string g_err;

// NVTX range around an API call (free when no profiler is attached).
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

// Checked mode (SPIRALPIR_CHECKED=1 when the context is created): every
// device allocation, and every buffer carved out of a query slot, is followed
// by a guard region filled with GUARD_FILL; the guards are verified after
// each synchronous call, so a kernel that writes past a buffer's end is
// reported (SP_ERR_DEVICE) with the buffer's name.
constexpr uint64_t GUARD_BYTES = 4096;
constexpr uint8_t GUARD_FILL = 0xA5;

struct Guard {
    uint8_t *p;
    uint64_t bytes;
    std::string what;
};

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? SP_ERR_NOMEM : SP_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

#define TRY(x)                 \
    do {                       \
        int rc_ = (x);         \
        if (rc_) return rc_;   \
    } while (0)

int ceil_log2(uint64_t x) {
    int v = 0;
    uint64_t p = 1;
    while (p < x) { p <<= 1; v++; }
    return v;
}

struct Db {
    DbLayout L{};
    uint32_t *d = nullptr;
    uint64_t bytes = 0;
};

struct Client {
    int n_left = 0, n_right = 0;
    uint32_t *keys = nullptr;   // one allocation: left | right | conv | pack
    const uint32_t *left = nullptr, *right = nullptr, *conv = nullptr, *pack = nullptr;
    uint64_t bytes = 0;
    uint64_t stamp = 0;         // last use (LRU)
};

struct Shape {
    int nu1 = 0, nu2 = 0, g = 0;
};

// Workspace of one query slot, sized for a maximal shape.
struct Slot {
    uint8_t *base = nullptr;
    uint64_t bytes = 0;
    QDesc q{};
    uint32_t *query32 = nullptr;
    uint64_t *query64 = nullptr;
    int client = -1, db = -1;
};

}  // namespace

namespace {

// One pipeline lane: a stream with its own workspace slots, descriptor
// arrays, events and pinned response staging.  The synchronous API runs on
// the main lane; the serving worker owns further lanes so that batches
// overlap on the GPU.
struct Lane {
    cudaStream_t st = nullptr;
    std::vector<Slot> slots;
    Shape slot_shape{};
    QDesc *d_qd = nullptr;       // [cap]
    QDesc *h_qd = nullptr;       // pinned mirror
    uint8_t *h_resp = nullptr;   // pinned responses [cap][response bytes]
    uint64_t *h_query = nullptr; // pinned query staging [cap][2 rows][2 primes][D]
    int *h_err = nullptr;        // pinned copy of d_err
    cudaEvent_t ev[6]{};
    bool ev_stages = false;             // the last run recorded ev[1..4] (stage timing)
    cudaEvent_t done = nullptr;
    // side stream of the Regev->GSW conversion, forked from the expansion
    // once its GSW-bit outputs are complete and joined before the multiply
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    int *d_err = nullptr;
    uint8_t *limbs = nullptr;           // tensor-core multiply workspace: selector digit
    uint64_t limb_bytes = 0;            // tiles, then the chunk output
    uint32_t *tc_out = nullptr;
    uint64_t tc_out_bytes = 0;
    SplitScratch split{};               // narrow fold levels split over CTAs
    uint64_t split_bytes = 0;
    int cap = 0;
    int staged = 0;
    bool busy = false;                  // serving: a batch is in flight
    std::vector<uint64_t> tickets;      // serving: tickets of that batch, slot order
    // instantiated pipeline graphs, keyed by the batch plan (see run_pipeline),
    // and how often each plan has run
    std::map<std::vector<int64_t>, cudaGraphExec_t> graphs;
    std::map<std::vector<int64_t>, int> plan_runs;
};

struct Pending {
    uint64_t ticket;
    int client_id, db_id;
    std::vector<uint64_t> query;        // copied at submission
    uint8_t *response;
    uint64_t response_len;
};

struct TicketState {
    int done = 0;
    int status = 0;
    uint8_t *response = nullptr;
    std::chrono::steady_clock::time_point submitted, completed;
};

}  // namespace

struct sp_ctx {
    sp_params p{};
    StageParams sp{};
    int device = 0;
    Lane main;
    cudaStream_t st = nullptr;      // main.st (stage entry points)
    int *d_err = nullptr;           // main.d_err
    TwiddleSet *d_tw = nullptr;
    uint32_t *d_neg1 = nullptr;     // [11][2][D] Montgomery form of NTT(x^(-2^r))
    uint8_t *h_stage = nullptr;     // pinned staging for database uploads
    uint64_t stage_bytes = 0;
    std::map<int, Db> dbs;
    std::map<int, Client> clients;
    uint64_t budget = 0, used = 0;
    uint64_t clock = 0;
    std::mutex mu;
    sp_stats_out stats{};
    // multiply variant chosen per (database id, size class ceil(log2 nq)):
    // 1 = per-query streaming kernel, 2 = batched integer kernel,
    // 3 = tensor-core kernel; and the per-query kernel's one-query time
    std::map<std::pair<int, int>, int> mul_choice;
    std::map<int, float> mul_single_ms;
    int mul_force = 0;          // 0 = autotune, 1..3 = force a variant
    // split schedule of the narrow launches (answer.cuh shifted_split) per
    // batch class (ceil log2 nq, deepest expansion, deepest fold): tuned on
    // first use unless forced; and the tuner's log
    int split_force = SP_SPLIT_AUTO;
    std::map<std::vector<int64_t>, int> plan_split;
    std::deque<std::string> tune_log;
    bool use_graphs = true;     // replay the answer pipeline as CUDA graphs
    // per-stage device time (sp_set_stage_timing): events between the
    // stages of each run, at about 5 us each; off, the stages follow one
    // another as dependent launches and only the run's total is timed
    bool stage_timing = false;
    // serving (continuous batching)
    std::vector<Lane *> lanes;
    std::thread worker;
    std::condition_variable cv;
    bool serving = false, stopping = false;
    std::deque<Pending> queue;
    std::map<uint64_t, TicketState> tickets;
    uint64_t next_ticket = 1;
    uint64_t served = 0, batches = 0;
    // checked mode: guard regions by allocation base, and the check's
    // device list and result word
    bool checked = false;
    std::map<uint8_t *, std::vector<Guard>> guards;
    uint64_t *d_guard_list = nullptr;
    int guard_list_cap = 0;
    uint32_t *d_guard_bad = nullptr;
};

namespace {

// Guard region [p, p + bytes) of allocation `base`, filled now.
int add_guard(sp_ctx *c, uint8_t *base, uint8_t *p, uint64_t bytes, const std::string &what) {
    CU(cudaMemset(p, GUARD_FILL, bytes));
    c->guards[base].push_back(Guard{p, bytes, what});
    return SP_OK;
}

// Device memory under the HBM budget (`bytes` counted; the guard region of
// the checked mode is not).
int alloc(sp_ctx *c, void **p, uint64_t bytes, const char *what = "device buffer") {
    if (c->budget && c->used + bytes > c->budget)
        return fail(SP_ERR_NOMEM, "HBM budget exceeded: need " + std::to_string(bytes) + " more bytes, " +
                                      std::to_string(c->budget - c->used) + " left");
    cudaError_t e = cudaMalloc(p, bytes + (c->checked ? GUARD_BYTES : 0));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(SP_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    c->used += bytes;
    if (c->checked) {
        uint8_t *b = (uint8_t *)*p;
        const int rc = add_guard(c, b, b + bytes, GUARD_BYTES, what);
        if (rc) {
            cudaFree(*p);
            *p = nullptr;
            c->used -= bytes;
            c->guards.erase(b);
            return rc;
        }
    }
    return SP_OK;
}

void release(sp_ctx *c, void *p, uint64_t bytes) {
    if (p) {
        cudaFree(p);
        c->used -= bytes;
        c->guards.erase((uint8_t *)p);
    }
}

// Checked mode: verify every guard region (waits for the device).
int verify_guards(sp_ctx *c) {
    if (!c->checked) return SP_OK;
    std::vector<uint64_t> list;
    std::vector<const Guard *> who;
    for (auto &kv : c->guards)
        for (const Guard &g : kv.second) {
            list.push_back((uint64_t)(uintptr_t)g.p);
            list.push_back(g.bytes);
            who.push_back(&g);
        }
    if (who.empty()) return SP_OK;
    CU(cudaDeviceSynchronize());
    if ((int)who.size() > c->guard_list_cap) {
        if (c->d_guard_list) cudaFree(c->d_guard_list);
        c->d_guard_list = nullptr;
        c->guard_list_cap = 0;
        CU(cudaMalloc(&c->d_guard_list, who.size() * 16));
        c->guard_list_cap = (int)who.size();
    }
    if (!c->d_guard_bad) CU(cudaMalloc(&c->d_guard_bad, sizeof(uint32_t)));
    CU(cudaMemcpy(c->d_guard_list, list.data(), list.size() * 8, cudaMemcpyHostToDevice));
    CU(cudaMemset(c->d_guard_bad, 0xff, sizeof(uint32_t)));
    CU(launch_check_guards(c->d_guard_list, (int)who.size(), GUARD_FILL, c->d_guard_bad, nullptr));
    uint32_t bad = 0;
    CU(cudaMemcpy(&bad, c->d_guard_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (bad != 0xffffffffu)
        return fail(SP_ERR_DEVICE, "device buffer overrun: the guard after " + who[bad]->what + " was overwritten");
    return SP_OK;
}

// Checked mode start-up: the check must pass, catch one flipped guard byte,
// and pass again once the byte is restored.
int guard_self_test(sp_ctx *c) {
    if (!c->checked || c->guards.empty()) return SP_OK;
    TRY(verify_guards(c));
    const Guard &g = c->guards.begin()->second.front();
    CU(cudaMemset(g.p + g.bytes / 2, 0, 1));
    const bool caught = verify_guards(c) == SP_ERR_DEVICE;
    CU(cudaMemset(g.p + g.bytes / 2, GUARD_FILL, 1));
    if (!caught) return fail(SP_ERR_DEVICE, "guard self-test: a flipped guard byte was not detected");
    return verify_guards(c);
}

int check_params(const sp_params *p) {
    if (!p) return fail(SP_ERR_INVALID, "params is NULL");
    if (p->n != 1 && p->n != 2 && p->n != 4)
        return fail(SP_ERR_UNSUPPORTED, "n must be 1, 2 or 4 (n*n plaintext polynomials per record, a power of two)");
    if (p->pt_bits < 1 || p->pt_bits > 8) return fail(SP_ERR_UNSUPPORTED, "pt_bits must be in [1, 8]");
    for (int t : {p->t_exp_left, p->t_exp_right, p->t_gsw, p->t_conv})
        if (t < 3 || t > 56) return fail(SP_ERR_UNSUPPORTED, "gadget lengths must be in [3, 56]");
    if (p->q2_bits < p->pt_bits + 2 || p->q2_bits > 32)
        return fail(SP_ERR_INVALID, "q2_bits must be in [pt_bits+2, 32]");
    if (p->max_batch < 1 || p->max_batch > 4096) return fail(SP_ERR_INVALID, "max_batch must be in [1, 4096]");
    return SP_OK;
}

Shape shape_of(const sp_ctx *c, int nu1, int nu2) {
    Shape s;
    s.nu1 = nu1;
    s.nu2 = nu2;
    s.g = ceil_log2((uint64_t)c->sp.t_gsw * nu2 + (1ull << nu1));
    return s;
}

// Carves a slot's workspace out of `base` (or only measures it, with
// base == nullptr); returns the bytes used.  One function for both, so the
// allocation always matches the carving.
// In checked mode every piece is followed by a guard gap (its alignment
// padding plus GUARD_BYTES), listed in `gaps` as (offset, bytes, name).
struct Gap {
    uint64_t off, bytes;
    const char *what;
};

uint64_t slot_layout(const sp_ctx *c, const Shape &s, uint8_t *base, Slot *sl, std::vector<Gap> *gaps = nullptr) {
    const uint64_t ct = 4ull * D * 4;   // NTT ciphertext bytes
    const int T = c->sp.T;
    uint64_t off = 0;
    auto take = [&](uint64_t x, const char *what) {
        uint8_t *r = base ? base + off : nullptr;
        const uint64_t end = off + ((x + 255) & ~255ull) + (c->checked ? GUARD_BYTES : 0);
        if (c->checked && gaps) gaps->push_back(Gap{off + x, end - off - x, what});
        off = end;
        return r;
    };
    uint32_t *query32 = (uint32_t *)take(ct, "slot query (u32)");
    uint64_t *query64 = (uint64_t *)take(ct * 2, "slot query (u64)");
    QDesc q{};
    q.query = query32;
    q.v[0] = (uint32_t *)take(ct << s.g, "slot expansion buffer 0");
    q.v[1] = (uint32_t *)take(ct << s.g, "slot expansion buffer 1");
    q.sel = (uint32_t *)take((uint64_t)D * 16 << s.nu1, "slot selectors");
    q.gsw_in = (uint32_t *)take(ct * s.nu2 * c->sp.t_gsw, "slot GSW-bit encodings");
    q.gsw = (uint32_t *)take((uint64_t)s.nu2 * 2 * 2 * c->sp.t_gsw * 2 * D * 4, "slot GSW ciphertexts");
    q.acc = (uint32_t *)take(((uint64_t)T * ct) << s.nu2, "slot multiply output");
    q.raw = (uint64_t *)take(((uint64_t)T * 2 * D * 8) << s.nu2, "slot fold buffer");
    q.resp = take(response_bytes(c->sp), "slot response bytes");
    if (sl) {
        sl->query32 = query32;
        sl->query64 = query64;
        sl->q = q;
    }
    return off;
}

uint64_t slot_bytes(const sp_ctx *c, const Shape &s) { return slot_layout(c, s, nullptr, nullptr); }

int carve(sp_ctx *c, Slot &sl, const Shape &s) {
    std::vector<Gap> gaps;
    slot_layout(c, s, sl.base, &sl, &gaps);
    for (const Gap &g : gaps) TRY(add_guard(c, sl.base, sl.base + g.off, g.bytes, g.what));
    return SP_OK;
}

void clear_graphs(Lane &L);

// Make sure there are `count` slots big enough for shape `need`.  Growing
// the shape reallocates every slot, which drops the lane's graphs (their
// input and response copies name slot buffers).
int ensure_slots(sp_ctx *c, Lane &L, const Shape &need, int count) {
    Shape s = L.slot_shape;
    bool grow = need.nu1 > s.nu1 || need.nu2 > s.nu2 || need.g > s.g;
    s.nu1 = std::max(s.nu1, need.nu1);
    s.nu2 = std::max(s.nu2, need.nu2);
    s.g = std::max(s.g, need.g);
    if (grow) {
        CU(cudaStreamSynchronize(L.st));
        clear_graphs(L);
        for (auto &sl : L.slots) release(c, sl.base, sl.bytes);
        L.slots.clear();
        L.staged = 0;
    }
    L.slot_shape = s;
    const uint64_t b = slot_bytes(c, s);
    while ((int)L.slots.size() < count) {
        Slot sl;
        int rc = alloc(c, (void **)&sl.base, b, "query slot");
        if (rc) return rc;
        sl.bytes = b;
        L.slots.push_back(sl);
        TRY(carve(c, L.slots.back(), s));
    }
    return SP_OK;
}

int ensure_staging(sp_ctx *c, uint64_t bytes) {
    if (c->stage_bytes >= bytes) return SP_OK;
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    CU(cudaMallocHost(&c->h_stage, bytes));
    c->stage_bytes = bytes;
    return SP_OK;
}

int lane_init(sp_ctx *c, Lane &L, int cap) {
    L.cap = cap;
    CU(cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking));
    CU(cudaStreamCreateWithFlags(&L.side, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&L.fork_ev, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&L.join_ev, cudaEventDisableTiming));
    for (auto &e : L.ev) CU(cudaEventCreate(&e));
    CU(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    TRY(alloc(c, (void **)&L.d_err, 16));
    TRY(alloc(c, (void **)&L.d_qd, sizeof(QDesc) * cap, "query descriptors"));
    CU(cudaMallocHost(&L.h_qd, sizeof(QDesc) * cap));
    memset(L.h_qd, 0, sizeof(QDesc) * cap);
    CU(cudaMallocHost(&L.h_resp, response_bytes(c->sp) * cap));
    CU(cudaMallocHost(&L.h_query, 4ull * D * 8 * cap));
    CU(cudaMallocHost(&L.h_err, 16));
    *L.h_err = 0;
    CU(cudaMemset(L.d_err, 0, 16));
    // split scratch: partial sums for up to 4 CTAs per SM, 4096 counters
    L.split.slots = 4 * sm_count();
    L.split.counter_slots = 4096;
    L.split_bytes = (uint64_t)L.split.slots * 4 * D * 4 + (uint64_t)L.split.counter_slots * 4;
    TRY(alloc(c, (void **)&L.split.part, L.split_bytes, "split partial sums"));
    L.split.counters = reinterpret_cast<uint32_t *>(L.split.part + (uint64_t)L.split.slots * 4 * D);
    CU(cudaMemset(L.split.counters, 0, (uint64_t)L.split.counter_slots * 4));
    return SP_OK;
}

// Graph instances bake in kernel arguments (descriptor array, database
// images, multiply workspace): drop them when one of those moves.
void clear_graphs(Lane &L) {
    for (auto &kv : L.graphs) cudaGraphExecDestroy(kv.second);
    L.graphs.clear();
    L.plan_runs.clear();
}

void lane_free(sp_ctx *c, Lane &L) {
    clear_graphs(L);
    if (L.st) cudaStreamSynchronize(L.st);
    for (auto &sl : L.slots) release(c, sl.base, sl.bytes);
    L.slots.clear();
    release(c, L.d_err, 16);
    release(c, L.d_qd, sizeof(QDesc) * L.cap);
    release(c, L.limbs, L.limb_bytes);
    L.limbs = nullptr;
    L.limb_bytes = 0;
    release(c, L.tc_out, L.tc_out_bytes);
    L.tc_out = nullptr;
    L.tc_out_bytes = 0;
    release(c, L.split.part, L.split_bytes);
    L.split = SplitScratch{};
    L.d_err = nullptr;
    L.d_qd = nullptr;
    if (L.h_qd) cudaFreeHost(L.h_qd);
    if (L.h_resp) cudaFreeHost(L.h_resp);
    if (L.h_query) cudaFreeHost(L.h_query);
    if (L.h_err) cudaFreeHost(L.h_err);
    L.h_qd = nullptr;
    L.h_resp = nullptr;
    L.h_query = nullptr;
    L.h_err = nullptr;
    for (auto &e : L.ev)
        if (e) cudaEventDestroy(e);
    if (L.done) cudaEventDestroy(L.done);
    if (L.side) cudaStreamSynchronize(L.side);
    if (L.fork_ev) cudaEventDestroy(L.fork_ev);
    if (L.join_ev) cudaEventDestroy(L.join_ev);
    if (L.side) cudaStreamDestroy(L.side);
    L.side = nullptr;
    L.fork_ev = L.join_ev = nullptr;
    if (L.st) cudaStreamDestroy(L.st);
    L.st = nullptr;
}

void clear_all_graphs(sp_ctx *c) {
    clear_graphs(c->main);
    for (Lane *l : c->lanes) clear_graphs(*l);
}

// A database id that is reloaded may change shape: forget its tuning.
void forget_db(sp_ctx *c, int db_id) {
    clear_all_graphs(c);
    for (auto it = c->mul_choice.begin(); it != c->mul_choice.end();)
        it = it->first.first == db_id ? c->mul_choice.erase(it) : std::next(it);
    c->mul_single_ms.erase(db_id);
}

// Wait for the GPU work of every lane (before freeing keys or databases).
int sync_all(sp_ctx *c) {
    if (c->main.st) CU(cudaStreamSynchronize(c->main.st));
    for (Lane *l : c->lanes)
        if (l->st) CU(cudaStreamSynchronize(l->st));
    return SP_OK;
}

void fill_desc(sp_ctx *c, QDesc &q, const Client &cl, const Db &db) {
    q.left = cl.left;
    q.right = cl.right;
    q.conv = cl.conv;
    q.pack = cl.pack;
    q.nu1 = db.L.nu1;
    q.nu2 = db.L.nu2;
    Shape s = shape_of(c, q.nu1, q.nu2);
    q.g = s.g;
    q.stop = ceil_log2((uint64_t)c->sp.t_gsw * q.nu2);
    q.capture = (q.stop > 0 && q.stop < q.g) ? q.stop : q.g - 1;
    q.active = 1;
}

int check_client_for(const sp_ctx *c, const Client &cl, const Db &db, int *need_left, int *need_right) {
    Shape s = shape_of(c, db.L.nu1, db.L.nu2);
    int stop = ceil_log2((uint64_t)c->sp.t_gsw * db.L.nu2);
    *need_left = s.g;
    *need_right = std::min(stop, s.g - 1) + 1;
    if (cl.n_left < *need_left || cl.n_right < *need_right)
        return fail(SP_ERR_INVALID, "client keys do not cover this database shape (need " +
                                        std::to_string(*need_left) + " left / " + std::to_string(*need_right) +
                                        " right expansion keys)");
    return SP_OK;
}

// Workspace of the tensor-core multiply for database layout `dl` (allocated
// once per lane, grown when needed, under the HBM budget).  Returns false
// when it does not fit.
bool ensure_limbs(sp_ctx *c, Lane &L, const DbLayout &dl) {
    const uint64_t need_l = tc_limb_bytes(dl), need_o = tc_out_bytes(dl);
    if (L.limb_bytes >= need_l && L.tc_out_bytes >= need_o) return true;
    if (L.limbs || L.tc_out) {
        if (cudaStreamSynchronize(L.st) != cudaSuccess) return false;
        clear_graphs(L);
    }
    if (L.limb_bytes < need_l) {
        release(c, L.limbs, L.limb_bytes);
        L.limbs = nullptr;
        L.limb_bytes = 0;
        if (alloc(c, (void **)&L.limbs, need_l, "tensor-core selector digits") != SP_OK) {
            g_err.clear();
            return false;
        }
        L.limb_bytes = need_l;
    }
    if (L.tc_out_bytes < need_o) {
        release(c, L.tc_out, L.tc_out_bytes);
        L.tc_out = nullptr;
        L.tc_out_bytes = 0;
        if (alloc(c, (void **)&L.tc_out, need_o, "tensor-core chunk output") != SP_OK) {
            g_err.clear();
            return false;
        }
        L.tc_out_bytes = need_o;
    }
    return true;
}

bool variant_available(sp_ctx *c, Lane &L, const Db &db, int nq, int variant) {
    switch (variant) {
        case 1: return true;
        case 2: return nq >= 2 && db_mul_batch_supported(db.L);
        case 3: return nq >= 2 && db_mul_tc_supported(db.L) && ensure_limbs(c, L, db.L);
        default: return false;
    }
}

// Enqueue the multiply of `nq` queries (descriptors qd) against `db`.
// pdl: the per-query kernel as a dependent launch of the previous kernel
cudaError_t launch_mul_variant(Lane &L, const Db &db, const QDesc *qd, int nq, int variant, bool pdl = false) {
    switch (variant) {
        case 2: return launch_db_mul_batch(db.d, db.L, qd, nq, L.st);
        case 3:
            for (int i = 0; i < nq; i += TC_MAX_Q) {
                const int k = std::min(TC_MAX_Q, nq - i);
                cudaError_t e = launch_db_mul_tc(db.d, db.L, qd + i, k, L.limbs, L.tc_out, L.d_err, L.st);
                if (e != cudaSuccess) return e;
            }
            return cudaSuccess;
        default: return launch_db_mul(db.d, db.L, qd, nq, L.d_err, L.st, pdl);
    }
}

// Autotuner of the first-dimension multiply.  The choice is kept per
// database and size class of the launch (ceil(log2 nq)).  The per-query
// streaming variant costs nq image passes, so it is estimated as nq times its
// one-query time, measured once per database; the best batched candidate
// (the tensor-core kernel where the shape allows it, else the integer batch
// kernel) runs once on the staged selectors and is timed with CUDA events.
// Outputs are identical; the timed runs are overwritten by the real one.
int time_variant(sp_ctx *c, Lane &L, const Db &db, const QDesc *qd, int nq, int variant, float *ms) {
    cudaEvent_t e[2];
    for (auto &x : e) CU(cudaEventCreate(&x));
    cudaError_t err = cudaEventRecord(e[0], L.st);
    if (!err) err = launch_mul_variant(L, db, qd, nq, variant);
    if (!err) err = cudaEventRecord(e[1], L.st);
    if (!err) err = cudaEventSynchronize(e[1]);
    if (!err) err = cudaEventElapsedTime(ms, e[0], e[1]);
    for (auto &x : e) cudaEventDestroy(x);
    if (err) return fail(SP_ERR_CUDA, std::string("multiply autotune: ") + cudaGetErrorString(err));
    return SP_OK;
}

// Whether choose_mul_variant answers without timing anything.
bool mul_choice_known(sp_ctx *c, Lane &L, int db_id, const Db &db, int nq) {
    if (c->mul_force && variant_available(c, L, db, nq, c->mul_force)) return true;
    if (nq < 2) return true;
    auto it = c->mul_choice.find(std::make_pair(db_id, ceil_log2((uint64_t)nq)));
    return it != c->mul_choice.end() && variant_available(c, L, db, nq, it->second);
}

int choose_mul_variant(sp_ctx *c, Lane &L, int db_id, const Db &db, const QDesc *qd, int nq, int *variant) {
    if (c->mul_force && variant_available(c, L, db, nq, c->mul_force)) {
        *variant = c->mul_force;
        return SP_OK;
    }
    if (nq < 2) {
        *variant = 1;
        return SP_OK;
    }
    const int cls = ceil_log2((uint64_t)nq);
    auto key = std::make_pair(db_id, cls);
    auto it = c->mul_choice.find(key);
    if (it != c->mul_choice.end() && variant_available(c, L, db, nq, it->second)) {
        *variant = it->second;
        return SP_OK;
    }
    const int cand = variant_available(c, L, db, nq, 3) ? 3 : (variant_available(c, L, db, nq, 2) ? 2 : 0);
    int best = 1;
    if (cand) {
        auto one = c->mul_single_ms.find(db_id);
        if (one == c->mul_single_ms.end()) {
            float ms1 = 0;
            TRY(time_variant(c, L, db, qd, 1, 1, &ms1));
            one = c->mul_single_ms.emplace(db_id, ms1).first;
        }
        float msb = 0;
        TRY(time_variant(c, L, db, qd, nq, cand, &msb));
        if (msb < one->second * nq) best = cand;
    }
    *variant = best;
    c->mul_choice[key] = best;
    return SP_OK;
}

// Uploads of an answer's inputs: the queries from the lane's pinned staging,
// converted to u32 residues, and the descriptors from L.h_qd.
cudaError_t enqueue_inputs(Lane &L, int nq, cudaStream_t st) {
    // one kernel reads the descriptors and queries from the pinned staging
    return launch_stage_in(L.h_qd, L.d_qd, L.h_query, nq, st);
}

// Autotuner of the narrow launches' split schedule (answer.cuh
// shifted_split).  The pipeline is idempotent from its staged inputs, so each
// candidate schedule runs it (on the batch at hand, after one untimed run),
// timed between the first and the last stage event; the fastest is kept for
// the batch class
// `key` = (ceil(log2 nq), deepest expansion, deepest fold); ties favour the
// rule, shift 0.  Every schedule gives identical residues.  The class and the
// candidate times go to the tuning log (sp_tuning_report).
template <typename Enqueue>
int tune_split(sp_ctx *c, Lane &L, const std::vector<int64_t> &key, Enqueue &enqueue, int *shift) {
    static const int cands[] = {0, -1, 1, SPLIT_NONE};
    float best_ms = 0;
    int best = 0;
    std::string msg = "plan class nq<=" + std::to_string(1ll << key[0]) + " g=" + std::to_string(key[1]) +
                      " nu2=" + std::to_string(key[2]) + ":";
    // one untimed run first (caches, lazily loaded kernels), then each
    // candidate timed once
    *shift = 0;
    CU(enqueue(false));
    for (int cand : cands) {
        *shift = cand;
        float ms = 0;
        CU(enqueue(false));
        CU(cudaEventSynchronize(L.ev[5]));
        CU(cudaEventElapsedTime(&ms, L.ev[0], L.ev[5]));
        msg += " shift " + (cand == SPLIT_NONE ? std::string("none") : std::to_string(cand)) + " " +
               std::to_string(ms).substr(0, 6) + " ms;";
        if (cand == 0 || ms < best_ms * 0.99f) {
            best_ms = ms;
            best = cand;
        }
    }
    *shift = best;
    c->plan_split[key] = best;
    msg += " chosen " + (best == SPLIT_NONE ? std::string("none") : std::to_string(best));
    c->tune_log.push_back(msg);
    while (c->tune_log.size() > 64) c->tune_log.pop_front();
    return SP_OK;
}

// Run the answer pipeline for queries in slots [0, nq) (descriptors in
// L.h_qd).  Without `io` the queries and descriptors are already on the
// device (sp_stage_query); with `io` the pipeline's first kernel reads them
// from the lane's pinned staging (L.h_query, L.h_qd: host memory the device
// addresses directly) and its last writes the responses to L.h_resp (the
// descriptors point there) and the error flag to L.h_err: no copies in the
// captured graph.
// Records the run's first and last events, and with stage timing the stage
// boundaries between them.
//
// The launches depend only on the batch plan: query count, the largest
// expansion depth / fold depth / conversion size, and per run of slots on one
// database its id, length and multiply variant.  The plan is the key of an
// instantiated CUDA graph of the whole pipeline (stage events included),
// captured the second time the plan runs (a capture costs more than one
// replay saves) and replayed afterwards; per-query inputs reach the kernels
// through the descriptor array, which is uploaded before each run.  A lane
// keeps at most 256 graphs; further plans run as plain launches.
int run_pipeline(sp_ctx *c, Lane &L, int nq, const std::vector<int> &db_of_slot, bool io) {
    cudaStream_t st = L.st;
    const StageParams &sp = c->sp;
    int max_g = 0, max_nu2 = 0, max_items = 0, fork_round = 0;
    for (int i = 0; i < nq; i++) {
        max_g = std::max(max_g, L.h_qd[i].g);
        max_nu2 = std::max(max_nu2, L.h_qd[i].nu2);
        max_items = std::max(max_items, L.h_qd[i].nu2 * sp.t_gsw);
        fork_round = std::max(fork_round, L.h_qd[i].capture);   // GSW-bit outputs complete after this round
    }
    // first-dimension multiply: consecutive slots of the same database share
    // a launch; variants are chosen (and autotuned) before any capture
    struct Group {
        int db_id, begin, count, variant;
    };
    std::vector<Group> groups;
    const bool timed = c->stage_timing;
    std::vector<int64_t> key = {nq, max_g, max_nu2, max_items, io ? 1 : 0, timed ? 1 : 0};
    uint64_t mul_bytes = 0;
    if (io) {
        // the autotuner times multiply launches on the staged descriptors:
        // upload them first when it will run
        bool known = true;
        for (int i = 0; i < nq;) {
            int j = i;
            while (j < nq && db_of_slot[j] == db_of_slot[i]) j++;
            known = known && mul_choice_known(c, L, db_of_slot[i], c->dbs.at(db_of_slot[i]), j - i);
            i = j;
        }
        if (!known) CU(enqueue_inputs(L, nq, st));
    }
    for (int i = 0; i < nq;) {
        int j = i;
        while (j < nq && db_of_slot[j] == db_of_slot[i]) j++;
        const Db &db = c->dbs.at(db_of_slot[i]);
        int variant = 1;
        TRY(choose_mul_variant(c, L, db_of_slot[i], db, L.d_qd + i, j - i, &variant));
        groups.push_back({db_of_slot[i], i, j - i, variant});
        key.insert(key.end(), {db_of_slot[i], j - i, variant});
        mul_bytes += db.L.image_bytes() + (uint64_t)(j - i) * ((uint64_t)db.L.rows * D * 16 +
                                                          (uint64_t)db.L.T * db.L.cols * 4 * D * 4);
        i = j;
    }
    // stage events are recorded as external event nodes so that a replayed
    // graph records them too.  Without stage timing there is no event between
    // stages and each stage's first kernel is a dependent launch of the
    // previous stage's last (its constant loads overlap that one's tail; a
    // per-query multiply streams the image before the selectors are ready)
    int cur_shift = 0;
    auto enqueue = [&](bool capturing) -> cudaError_t {
        const unsigned ev_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
        // a captured graph holds events only with stage timing; otherwise the
        // run's first and last events go on the stream around the graph
        const bool run_ev = timed || !capturing;
        cudaError_t e = io ? enqueue_inputs(L, nq, st) : cudaSuccess;
        if (!e && run_ev) e = cudaEventRecordWithFlags(L.ev[0], st, ev_flags);
        for (int r = 0; r < max_g && !e; r++) {
            e = launch_expand_round(L.d_qd, nq, r, 2 << r, sp, c->d_tw, c->d_neg1, &L.split, st, cur_shift);
            if (!e && r == fork_round) {
                // the conversion needs only the GSW-bit encodings: run it on
                // the side stream, overlapping the remaining rounds
                e = cudaEventRecord(L.fork_ev, st);
                if (!e) e = cudaStreamWaitEvent(L.side, L.fork_ev, 0);
                if (!e) e = launch_regev_to_gsw(L.d_qd, nq, max_items, sp, c->d_tw, L.side);
                if (!e) e = cudaEventRecord(L.join_ev, L.side);
            }
        }
        if (!e && timed) e = cudaEventRecordWithFlags(L.ev[1], st, ev_flags);
        // the folds need the GSW ciphertexts: join the conversion here, where
        // it has long finished (it overlaps the last expansion rounds)
        if (!e) e = cudaStreamWaitEvent(st, L.join_ev, 0);
        if (!e && timed) e = cudaEventRecordWithFlags(L.ev[2], st, ev_flags);   // conversion past the expansion
        for (size_t k = 0; k < groups.size() && !e; k++) {
            const Group &gr = groups[k];
            e = launch_mul_variant(L, c->dbs.at(gr.db_id), L.d_qd + gr.begin, gr.count, gr.variant, !timed && k == 0);
        }
        if (!e && timed) e = cudaEventRecordWithFlags(L.ev[3], st, ev_flags);
        if (!e) e = launch_acc_to_raw(L.d_qd, nq, sp.T * (2 << max_nu2), sp, c->d_tw, st, !timed);
        for (int lvl = 0; lvl < max_nu2 && !e; lvl++)
            e = launch_fold_level(L.d_qd, nq, lvl, sp.T << (max_nu2 - 1 - lvl), sp, c->d_tw, &L.split, st, cur_shift,
                                  true);
        if (!e && timed) e = cudaEventRecordWithFlags(L.ev[4], st, ev_flags);
        // with host I/O the responses (descriptors point into the pinned
        // staging) and the error flag go to host memory from the kernel
        if (!e) e = launch_pack(L.d_qd, nq, sp, c->d_tw, &L.split, st, cur_shift, io ? L.d_err : nullptr,
                                io ? L.h_err : nullptr, !timed);
        if (!e && run_ev) e = cudaEventRecordWithFlags(L.ev[5], st, ev_flags);
        return e;
    };
    // split schedule: forced, tuned earlier for this batch class, or tuned
    // now.  The class is what shapes the narrow launches: the batch size
    // class ceil(log2 nq) and the deepest expansion and fold (so serving,
    // where almost every batch mixes databases differently, tunes once per
    // class, not per batch)
    if (c->split_force != SP_SPLIT_AUTO) {
        cur_shift = c->split_force;
    } else {
        const std::vector<int64_t> cls = {ceil_log2((uint64_t)nq), max_g, max_nu2};
        auto ps = c->plan_split.find(cls);
        if (ps != c->plan_split.end()) {
            cur_shift = ps->second;
        } else {
            TRY(tune_split(c, L, cls, enqueue, &cur_shift));
        }
    }
    key.push_back(cur_shift);
    auto it = L.graphs.find(key);
    bool replay = c->use_graphs && it != L.graphs.end();
    if (c->use_graphs && !replay && L.graphs.size() < 256) {
        if (L.plan_runs.size() > 4096) L.plan_runs.clear();
        replay = ++L.plan_runs[key] >= 2;
    }
    if (replay) {
        if (it == L.graphs.end()) {
            cudaGraph_t graph = nullptr;
            CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            const cudaError_t e = enqueue(true);
            const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();
                return fail(SP_ERR_CUDA, std::string("pipeline capture: ") +
                                             cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            cudaGraphExec_t exec = nullptr;
            const cudaError_t e3 = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e3 != cudaSuccess) return fail(SP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
            it = L.graphs.emplace(key, exec).first;
        }
        if (!timed) CU(cudaEventRecord(L.ev[0], st));
        CU(cudaGraphLaunch(it->second, st));
        if (!timed) CU(cudaEventRecord(L.ev[5], st));
    } else {
        CU(enqueue(false));
    }
    L.ev_stages = timed;
    // expansion rounds, conversion, output to raw, fold levels, pack, and
    // the staging kernel of runs with host I/O
    uint64_t launches = (uint64_t)max_g + 1 + 1 + (uint64_t)max_nu2 + 1 + (io ? 1 : 0);
    for (const Group &gr : groups) {
        c->stats.db_mul_by_variant[gr.variant - 1]++;
        launches += gr.variant == 3 ? (uint64_t)tc_launches(c->dbs.at(gr.db_id).L) * ((gr.count + TC_MAX_Q - 1) / TC_MAX_Q)
                                    : 1;
    }
    c->stats.launches += launches;
    c->stats.db_mul_calls += groups.size();
    c->stats.db_mul_bytes += mul_bytes;
    c->stats.answers += nq;
    return SP_OK;
}

int collect_stats(sp_ctx *c, Lane &L) {
    float ms[5] = {0, 0, 0, 0, 0}, tot;
    if (L.ev_stages)
        for (int i = 0; i < 5; i++) CU(cudaEventElapsedTime(&ms[i], L.ev[i], L.ev[i + 1]));
    CU(cudaEventElapsedTime(&tot, L.ev[0], L.ev[5]));
    c->stats.ms_expand += ms[0];
    c->stats.ms_convert += ms[1];
    c->stats.ms_db_mul += ms[2];
    c->stats.ms_fold += ms[3];
    c->stats.ms_pack += ms[4];
    c->stats.ms_total += tot;
    return SP_OK;
}

// The device error flag as last copied to L.h_err (the copy has completed):
// a bounded wait that ran out is reported once and the flag cleared.
int take_device_err(sp_ctx *c, Lane &L) {
    const int h = *L.h_err;
    if (h) {
        *L.h_err = 0;
        CU(cudaMemsetAsync(L.d_err, 0, sizeof(int), L.st));
        return fail(SP_ERR_DEVICE, "a device-side bounded wait ran out (code " + std::to_string(h) + ")");
    }
    return verify_guards(c);
}

int check_device_err(sp_ctx *c, Lane &L) {
    CU(cudaMemcpyAsync(L.h_err, L.d_err, sizeof(int), cudaMemcpyDeviceToHost, L.st));
    CU(cudaStreamSynchronize(L.st));
    return take_device_err(c, L);
}

// Temporary device buffer for stage calls (freed on scope exit).
struct Tmp {
    sp_ctx *c;
    void *p = nullptr;
    uint64_t b = 0;
    explicit Tmp(sp_ctx *ctx) : c(ctx) {}
    int get(uint64_t bytes) {
        b = bytes;
        return alloc(c, &p, bytes ? bytes : 16, "stage call buffer");
    }
    ~Tmp() { release(c, p, b ? b : 16); }
    template <typename T> T *as() const { return (T *)p; }
};

}  // namespace

// ===================================================================== API
extern "C" {

int sp_serve_stop(sp_ctx *c);

int sp_last_error(char *buf, size_t len) {
    if (!buf || !len) return SP_ERR_INVALID;
    snprintf(buf, len, "%s", g_err.c_str());
    return SP_OK;
}

int sp_ctx_create(const sp_params *params, uint64_t hbm_budget_bytes, sp_ctx **out) {
    if (!out) return fail(SP_ERR_INVALID, "out is NULL");
    *out = nullptr;
    TRY(check_params(params));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SP_ERR_CUDA, "no CUDA device");
    }
    sp_ctx *c = new sp_ctx();
    c->p = *params;
    c->sp.n = params->n;
    c->sp.T = params->n * params->n;
    c->sp.pt_bits = params->pt_bits;
    c->sp.q2_bits = params->q2_bits;
    c->sp.t_left = params->t_exp_left;
    c->sp.t_right = params->t_exp_right;
    c->sp.t_gsw = params->t_gsw;
    c->sp.t_conv = params->t_conv;
    c->budget = hbm_budget_bytes;
    if (const char *ck = std::getenv("SPIRALPIR_CHECKED")) c->checked = ck[0] && ck[0] != '0';
    auto bail = [&](int rc) {
        sp_ctx_destroy(c);
        return rc;
    };
    if (cudaGetDevice(&c->device) != cudaSuccess) return bail(fail(SP_ERR_CUDA, "cudaGetDevice failed"));
    int rc = lane_init(c, c->main, params->max_batch);
    if (rc) return bail(rc);
    c->st = c->main.st;
    c->d_err = c->main.d_err;
    rc = alloc(c, (void **)&c->d_tw, sizeof(TwiddleSet), "twiddle tables");
    if (!rc) rc = alloc(c, (void **)&c->d_neg1, (uint64_t)LOGD * 2 * D * 4, "x^-2^r factors");
    if (rc) return bail(rc);
    // constant tables
    std::vector<TwiddleSet> tw(1);
    build_twiddles_host(tw.data());
    std::vector<uint32_t> neg1((size_t)LOGD * 2 * D);
    const uint32_t psi[2] = {66687u, 158221u};
    for (int r = 0; r < LOGD; r++)
        for (int k = 0; k < 2; k++) {
            const Prime pr = prime_of(k);
            const uint64_t p = pr.p;
            const uint64_t psi_inv = powmod_c(psi[k], 4095, p);
            for (int z = 0; z < D; z++) {
                uint32_t rz = 0, x = z;
                for (int b = 0; b < LOGD; b++) { rz = (rz << 1) | (x & 1); x >>= 1; }
                // slot z of x^(-2^r): psi^(-(2*brev(z)+1) * 2^r)
                uint64_t v = powmod_c(psi_inv, ((uint64_t)(2 * rz + 1) << r) % 4096, p);
                neg1[((size_t)r * 2 + k) * D + z] = (uint32_t)(v * pr.two32 % p);
            }
        }
    if (cudaMemcpy(c->d_tw, tw.data(), sizeof(TwiddleSet), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c->d_neg1, neg1.data(), neg1.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(SP_ERR_CUDA, "constant upload failed"));
    rc = guard_self_test(c);
    if (rc) return bail(rc);
    *out = c;
    return SP_OK;
}

int sp_ctx_destroy(sp_ctx *c) {
    if (!c) return SP_OK;
    sp_serve_stop(c);
    sync_all(c);
    for (auto &kv : c->dbs) release(c, kv.second.d, kv.second.bytes);
    for (auto &kv : c->clients) release(c, kv.second.keys, kv.second.bytes);
    lane_free(c, c->main);
    release(c, c->d_tw, sizeof(TwiddleSet));
    release(c, c->d_neg1, (uint64_t)LOGD * 2 * D * 4);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->d_guard_list) cudaFree(c->d_guard_list);
    if (c->d_guard_bad) cudaFree(c->d_guard_bad);
    delete c;
    return SP_OK;
}

int sp_response_bytes(const sp_ctx *c, uint64_t *bytes) {
    if (!c || !bytes) return fail(SP_ERR_INVALID, "NULL argument");
    *bytes = response_bytes(c->sp);
    return SP_OK;
}

int sp_wait_probe(sp_ctx *c, int32_t limit_ms) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    if (limit_ms < 1 || limit_ms > 1000) return fail(SP_ERR_INVALID, "limit_ms must be in [1, 1000]");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_wait_probe");
    CU(launch_wait_probe(c->main.d_err, (uint64_t)limit_ms * 1000000ull, c->main.st));
    return check_device_err(c, c->main);
}

int sp_check_guards(sp_ctx *c, int32_t *checked) {
    if (!c || !checked) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    *checked = c->checked ? 1 : 0;
    return verify_guards(c);
}

int sp_hbm_used(const sp_ctx *c, uint64_t *bytes) {
    if (!c || !bytes) return fail(SP_ERR_INVALID, "NULL argument");
    *bytes = c->used;
    return SP_OK;
}

// ------------------------------------------------------------- databases
static int db_check_shape(sp_ctx *c, int nu1, int nu2) {
    if (nu1 < 1 || nu1 > 14 || nu2 < 1 || nu2 > 14) return fail(SP_ERR_INVALID, "nu1/nu2 out of range");
    if (shape_of(c, nu1, nu2).g > LOGD)
        return fail(SP_ERR_UNSUPPORTED, "expansion needs more than 11 rounds (t_gsw*nu2 + 2^nu1 > 2048)");
    // the expansion interleaves 2^nu1 selectors (even outputs) with t_gsw*nu2
    // GSW-bit encodings (odd outputs) in 2^g outputs: both halves must fit
    if (((uint64_t)c->sp.t_gsw * nu2 << 1) > (1ull << shape_of(c, nu1, nu2).g))
        return fail(SP_ERR_UNSUPPORTED, "t_gsw*nu2 GSW-bit encodings do not fit the odd expansion outputs "
                                        "(needs 2^nu1 >= t_gsw*nu2)");
    DbLayout L = make_db_layout(c->sp.T, nu1, nu2);
    // an image unit (rows packed rows of cbp 28-bit places) must be a whole
    // number of 16-byte copy granules
    if ((uint64_t)L.rows * L.cbp < 32)
        return fail(SP_ERR_UNSUPPORTED, "database unit smaller than 32 residue places (2^nu1 * combo block < 32)");
    return SP_OK;
}

static int db_alloc(sp_ctx *c, int db_id, int nu1, int nu2, Db &db) {
    TRY(db_check_shape(c, nu1, nu2));
    if (c->dbs.count(db_id)) {
        TRY(sync_all(c));
        forget_db(c, db_id);
        release(c, c->dbs[db_id].d, c->dbs[db_id].bytes);
        c->dbs.erase(db_id);
    }
    db.L = make_db_layout(c->sp.T, nu1, nu2);
    db.bytes = db.L.image_bytes();
    return alloc(c, (void **)&db.d, db.bytes, "database image");
}

int sp_db_load_plain(sp_ctx *c, int32_t db_id, const uint8_t *records, uint64_t n_records, int32_t nu1,
                     int32_t nu2) {
    if (!c || !records) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_load_plain");
    if (n_records != (1ull << (nu1 + nu2))) return fail(SP_ERR_INVALID, "n_records must be 2^(nu1+nu2)");
    Db db;
    TRY(db_alloc(c, db_id, nu1, nu2, db));
    // stream the records through a pinned staging buffer in chunks of whole
    // packed groups (multiples of 8 records); each chunk is transformed into
    // `ntt` and packed into the image
    const uint64_t rec_bytes = (uint64_t)c->sp.T * D;
    const uint64_t chunk_recs =
        std::min<uint64_t>(n_records, std::max<uint64_t>(8, (4ull << 20) / rec_bytes / 8 * 8));
    Tmp dev(c), ntt(c);
    int rc = dev.get(2 * chunk_recs * rec_bytes);
    if (!rc) rc = ntt.get(chunk_recs * c->sp.T * 2 * D * 4);
    if (!rc) rc = ensure_staging(c, 2 * chunk_recs * rec_bytes);
    if (rc) {
        release(c, db.d, db.bytes);
        return rc;
    }
    int buf = 0;
    cudaEvent_t done[2];
    cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming);
    cudaEventRecord(done[0], c->st);
    cudaEventRecord(done[1], c->st);
    cudaError_t err = cudaSuccess;
    for (uint64_t r0 = 0; r0 < n_records && err == cudaSuccess; r0 += chunk_recs, buf ^= 1) {
        const uint64_t cnt = std::min(chunk_recs, n_records - r0);
        uint8_t *hs = c->h_stage + buf * chunk_recs * rec_bytes;
        uint8_t *ds = dev.as<uint8_t>() + buf * chunk_recs * rec_bytes;
        cudaEventSynchronize(done[buf]);   // staging half free again
        memcpy(hs, records + r0 * rec_bytes, cnt * rec_bytes);
        err = cudaMemcpyAsync(ds, hs, cnt * rec_bytes, cudaMemcpyHostToDevice, c->st);
        if (err == cudaSuccess)
            err = launch_db_encode(ds, r0, cnt, c->sp.pt_bits, db.L, ntt.as<uint32_t>(), db.d, c->d_tw, c->st);
        cudaEventRecord(done[buf], c->st);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(c->st);
    cudaEventDestroy(done[0]);
    cudaEventDestroy(done[1]);
    if (err != cudaSuccess) {
        release(c, db.d, db.bytes);
        return fail(SP_ERR_CUDA, std::string("database encode: ") + cudaGetErrorString(err));
    }
    c->dbs[db_id] = db;
    return SP_OK;
}

int sp_db_load_ntt(sp_ctx *c, int32_t db_id, const uint32_t *planes, int32_t nu1, int32_t nu2) {
    if (!c || !planes) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_load_ntt");
    Db db;
    TRY(db_alloc(c, db_id, nu1, nu2, db));
    Tmp dev(c);
    int rc = dev.get(db.L.words * 8);
    if (rc) {
        release(c, db.d, db.bytes);
        return rc;
    }
    cudaError_t err = cudaMemcpyAsync(dev.p, planes, db.L.words * 8, cudaMemcpyHostToDevice, c->st);
    if (err == cudaSuccess) err = launch_db_import(dev.as<uint32_t>(), db.L, db.d, c->st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(c->st);
    if (err != cudaSuccess) {
        release(c, db.d, db.bytes);
        return fail(SP_ERR_CUDA, std::string("database import: ") + cudaGetErrorString(err));
    }
    c->dbs[db_id] = db;
    return SP_OK;
}

// ------------------------------------------------------------ checkpoints
namespace {

struct ImageHeader {
    char magic[8];          // "SPIRDB1"
    uint32_t version;       // 1
    uint32_t layout;        // 2: 28-bit residues, 8 per 7 words, [prime][z][combo block][row][combo]
    int32_t n, pt_bits, nu1, nu2;
    uint32_t d, q1, q2;
    uint32_t reserved;
    uint64_t image_bytes;
    uint64_t fnv;           // FNV-1a 64 over the image's 64-bit words
};
static_assert(sizeof(ImageHeader) == 64, "image header is 64 bytes");

constexpr char IMAGE_MAGIC[8] = {'S', 'P', 'I', 'R', 'D', 'B', '1', 0};
constexpr uint64_t FNV_OFFSET = 1469598103934665603ull, FNV_PRIME = 1099511628211ull;

// FNV-1a over little-endian 64-bit words (n is a multiple of 8).
uint64_t fnv1a(uint64_t h, const uint8_t *p, uint64_t n) {
    for (uint64_t i = 0; i + 8 <= n; i += 8) {
        uint64_t w;
        memcpy(&w, p + i, 8);
        h = (h ^ w) * FNV_PRIME;
    }
    return h;
}

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

constexpr uint64_t CKPT_CHUNK = 64ull << 20;

}  // namespace

int sp_db_save(sp_ctx *c, int32_t db_id, const char *path) {
    if (!c || !path) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_save");
    auto it = c->dbs.find(db_id);
    if (it == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id");
    const Db &db = it->second;
    TRY(sync_all(c));
    TRY(ensure_staging(c, CKPT_CHUNK));
    File out;
    out.f = fopen(path, "wb");
    if (!out.f) return fail(SP_ERR_IO, std::string("cannot open ") + path + " for writing");
    ImageHeader h{};
    memcpy(h.magic, IMAGE_MAGIC, 8);
    h.version = 1;
    h.layout = 2;
    h.n = c->sp.n;
    h.pt_bits = c->sp.pt_bits;
    h.nu1 = db.L.nu1;
    h.nu2 = db.L.nu2;
    h.d = D;
    h.q1 = QP0;
    h.q2 = QP1;
    h.image_bytes = db.bytes;
    h.fnv = FNV_OFFSET;
    // header first (checksum patched in at the end)
    if (fwrite(&h, sizeof h, 1, out.f) != 1) return fail(SP_ERR_IO, std::string("cannot write ") + path);
    const uint8_t *src = reinterpret_cast<const uint8_t *>(db.d);
    for (uint64_t off = 0; off < db.bytes; off += CKPT_CHUNK) {
        const uint64_t n = std::min(CKPT_CHUNK, db.bytes - off);
        CU(cudaMemcpyAsync(c->h_stage, src + off, n, cudaMemcpyDeviceToHost, c->st));
        CU(cudaStreamSynchronize(c->st));
        h.fnv = fnv1a(h.fnv, c->h_stage, n);
        if (fwrite(c->h_stage, 1, n, out.f) != n) return fail(SP_ERR_IO, std::string("cannot write ") + path);
    }
    if (fseek(out.f, 0, SEEK_SET) != 0 || fwrite(&h, sizeof h, 1, out.f) != 1 || fflush(out.f) != 0)
        return fail(SP_ERR_IO, std::string("cannot write ") + path);
    return SP_OK;
}

int sp_db_restore(sp_ctx *c, int32_t db_id, const char *path) {
    if (!c || !path) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_restore");
    File in;
    in.f = fopen(path, "rb");
    if (!in.f) return fail(SP_ERR_IO, std::string("cannot open ") + path);
    ImageHeader h{};
    if (fread(&h, sizeof h, 1, in.f) != 1 || memcmp(h.magic, IMAGE_MAGIC, 8) != 0 || h.version != 1 ||
        h.layout != 2)
        return fail(SP_ERR_INVALID, std::string(path) + " is not a database image of this library");
    if (h.d != (uint32_t)D || h.q1 != QP0 || h.q2 != QP1 || h.n != c->sp.n || h.pt_bits != c->sp.pt_bits)
        return fail(SP_ERR_INVALID, "database image was written for other ring or plaintext parameters");
    const DbLayout L = make_db_layout(c->sp.T, h.nu1, h.nu2);
    if (h.nu1 < 1 || h.nu2 < 1 || h.nu1 > 14 || h.nu2 > 14 || h.image_bytes != L.image_bytes())
        return fail(SP_ERR_INVALID, "database image header does not describe a valid shape");
    Db db;
    TRY(db_alloc(c, db_id, h.nu1, h.nu2, db));
    int rc = ensure_staging(c, CKPT_CHUNK);
    uint64_t fnv = FNV_OFFSET;
    uint8_t *dst = reinterpret_cast<uint8_t *>(db.d);
    for (uint64_t off = 0; off < db.bytes && !rc; off += CKPT_CHUNK) {
        const uint64_t n = std::min(CKPT_CHUNK, db.bytes - off);
        if (fread(c->h_stage, 1, n, in.f) != n) {
            rc = fail(SP_ERR_INVALID, std::string(path) + " is shorter than its header says");
            break;
        }
        fnv = fnv1a(fnv, c->h_stage, n);
        cudaError_t e = cudaMemcpyAsync(dst + off, c->h_stage, n, cudaMemcpyHostToDevice, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) rc = fail(SP_ERR_CUDA, std::string("database restore: ") + cudaGetErrorString(e));
    }
    if (!rc && fnv != h.fnv) rc = fail(SP_ERR_INVALID, std::string(path) + ": image checksum mismatch");
    if (rc) {
        release(c, db.d, db.bytes);
        return rc;
    }
    c->dbs[db_id] = db;
    return SP_OK;
}

int sp_db_unload(sp_ctx *c, int32_t db_id) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_unload");
    auto it = c->dbs.find(db_id);
    if (it == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id");
    TRY(sync_all(c));
    forget_db(c, db_id);
    release(c, it->second.d, it->second.bytes);
    c->dbs.erase(it);
    return SP_OK;
}

// ----------------------------------------------------------------- clients
static int evict_lru(sp_ctx *c, uint64_t need) {
    while (c->budget && c->used + need > c->budget && !c->clients.empty()) {
        auto victim = c->clients.begin();
        for (auto it = c->clients.begin(); it != c->clients.end(); ++it)
            if (it->second.stamp < victim->second.stamp) victim = it;
        release(c, victim->second.keys, victim->second.bytes);
        c->clients.erase(victim);
    }
    return SP_OK;
}

}  // extern "C"

namespace {

// Registers client keys: `fill` enqueues on c->st the copies of the key
// words into `u` (u64 staging in the device key layout: left | right | conv |
// pack); with `seed`, row 0 of every key matrix is then regenerated on the
// device from it (csrc/seeded.cu) instead of being copied.
template <typename Fill>
int set_keys_impl(sp_ctx *c, int32_t client_id, int32_t n_left, int32_t n_right, Fill fill, const SeedKey *seed) {
    if (n_left < 1 || n_left > LOGD || n_right < 1 || n_right > LOGD)
        return fail(SP_ERR_INVALID, "expansion key counts must be in [1, 11]");
    const StageParams &s = c->sp;
    const uint64_t P = 2ull * D;   // words per NTT poly
    const uint64_t wl = (uint64_t)n_left * 2 * s.t_left * P, wr = (uint64_t)n_right * 2 * s.t_right * P;
    const uint64_t wc = 2ull * 2 * s.t_conv * P, wp = (uint64_t)s.n * (s.n + 1) * s.t_conv * P;
    const uint64_t words = wl + wr + wc + wp;
    TRY(sync_all(c));
    auto old = c->clients.find(client_id);
    if (old != c->clients.end()) {
        release(c, old->second.keys, old->second.bytes);
        c->clients.erase(old);
    }
    evict_lru(c, words * 4 + words * 8);
    Client cl;
    cl.n_left = n_left;
    cl.n_right = n_right;
    cl.bytes = words * 4;
    TRY(alloc(c, (void **)&cl.keys, cl.bytes, "client keys"));
    Tmp up(c);
    int rc = up.get(words * 8);
    if (rc) {
        release(c, cl.keys, cl.bytes);
        return rc;
    }
    uint64_t *u = up.as<uint64_t>();
    // seeded: the row-0 planes are regenerated below; clear them so that the
    // conversion reads defined words
    cudaError_t e = seed ? cudaMemsetAsync(u, 0, words * 8, c->st) : cudaSuccess;
    if (e == cudaSuccess) e = fill(u, wl, wr, wc);
    if (e == cudaSuccess) e = launch_narrow(u, cl.keys, words / D, true, c->st);
    if (e == cudaSuccess && seed) {
        SeedRowMap m{n_left, s.t_left, n_right, s.t_right, s.t_conv, s.n,
                     (uint32_t)(n_left * s.t_left + n_right * s.t_right + 2 * s.t_conv + s.n * s.t_conv)};
        e = launch_seed_rows(*seed, m, cl.keys, c->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
        release(c, cl.keys, cl.bytes);
        return fail(SP_ERR_CUDA, std::string("key upload: ") + cudaGetErrorString(e));
    }
    cl.left = cl.keys;
    cl.right = cl.keys + wl;
    cl.conv = cl.keys + wl + wr;
    cl.pack = cl.keys + wl + wr + wc;
    cl.stamp = ++c->clock;
    c->clients[client_id] = cl;
    return SP_OK;
}

}  // namespace

extern "C" {

int sp_client_set_keys(sp_ctx *c, int32_t client_id, const uint64_t *exp_left, int32_t n_left,
                       const uint64_t *exp_right, int32_t n_right, const uint64_t *conv, const uint64_t *pack) {
    if (!c || !exp_left || !exp_right || !conv || !pack) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_client_set_keys");
    const StageParams &s = c->sp;
    auto fill = [&](uint64_t *u, uint64_t wl, uint64_t wr, uint64_t wc) {
        const uint64_t wp = (uint64_t)s.n * (s.n + 1) * s.t_conv * 2 * D;
        const uint64_t *src[4] = {exp_left, exp_right, conv, pack};
        const uint64_t cnt[4] = {wl, wr, wc, wp};
        uint64_t off = 0;
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < 4 && e == cudaSuccess; i++) {
            e = cudaMemcpyAsync(u + off, src[i], cnt[i] * 8, cudaMemcpyHostToDevice, c->st);
            off += cnt[i];
        }
        return e;
    };
    return set_keys_impl(c, client_id, n_left, n_right, fill, nullptr);
}

int sp_client_set_keys_seeded(sp_ctx *c, int32_t client_id, const uint8_t *seed, const uint64_t *left_rest,
                              int32_t n_left, const uint64_t *right_rest, int32_t n_right, const uint64_t *conv_rest,
                              const uint64_t *pack_rest) {
    if (!c || !seed || !left_rest || !right_rest || !conv_rest || !pack_rest)
        return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_client_set_keys_seeded");
    const StageParams &s = c->sp;
    SeedKey key;
    for (int i = 0; i < 8; i++)
        key.w[i] = (uint32_t)seed[4 * i] | (uint32_t)seed[4 * i + 1] << 8 | (uint32_t)seed[4 * i + 2] << 16 |
                   (uint32_t)seed[4 * i + 3] << 24;
    // each matrix's rows below row 0 go to their place in the full layout
    auto fill = [&](uint64_t *u, uint64_t wl, uint64_t wr, uint64_t wc) {
        const uint64_t P = 2ull * D;
        cudaError_t e = cudaSuccess;
        for (int r = 0; r < n_left && e == cudaSuccess; r++)
            e = cudaMemcpyAsync(u + ((uint64_t)r * 2 + 1) * s.t_left * P, left_rest + (uint64_t)r * s.t_left * P,
                                (uint64_t)s.t_left * P * 8, cudaMemcpyHostToDevice, c->st);
        for (int r = 0; r < n_right && e == cudaSuccess; r++)
            e = cudaMemcpyAsync(u + wl + ((uint64_t)r * 2 + 1) * s.t_right * P, right_rest + (uint64_t)r * s.t_right * P,
                                (uint64_t)s.t_right * P * 8, cudaMemcpyHostToDevice, c->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(u + wl + wr + 2ull * s.t_conv * P, conv_rest, 2ull * s.t_conv * P * 8,
                                cudaMemcpyHostToDevice, c->st);
        for (int r = 0; r < s.n && e == cudaSuccess; r++)
            e = cudaMemcpyAsync(u + wl + wr + wc + ((uint64_t)r * (s.n + 1) + 1) * s.t_conv * P,
                                pack_rest + (uint64_t)r * s.n * s.t_conv * P, (uint64_t)s.n * s.t_conv * P * 8,
                                cudaMemcpyHostToDevice, c->st);
        return e;
    };
    return set_keys_impl(c, client_id, n_left, n_right, fill, &key);
}

int sp_client_evict(sp_ctx *c, int32_t client_id) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_client_evict");
    auto it = c->clients.find(client_id);
    if (it == c->clients.end()) return fail(SP_ERR_NOT_FOUND, "unknown client id");
    TRY(sync_all(c));
    release(c, it->second.keys, it->second.bytes);
    c->clients.erase(it);
    return SP_OK;
}

// --------------------------------------------------------------- answering
// Validate requests and fill slots [0, n) with descriptors (queries copied
// in from host memory).  Requests are ordered by database so that each
// database's multiply is one launch.
static int prepare(sp_ctx *c, Lane &L, int n, sp_request *reqs, std::vector<int> &order, std::vector<int> &db_of_slot) {
    if (n < 1 || n > L.cap) return fail(SP_ERR_INVALID, "batch size out of range");
    Shape need{};
    for (int i = 0; i < n; i++) {
        sp_request &r = reqs[i];
        if (!r.query || !r.response) return fail(SP_ERR_INVALID, "NULL query or response");
        if (r.response_len < response_bytes(c->sp)) return fail(SP_ERR_INVALID, "response buffer too small");
        auto ci = c->clients.find(r.client_id);
        if (ci == c->clients.end()) return fail(SP_ERR_NOT_FOUND, "unknown client id " + std::to_string(r.client_id));
        auto di = c->dbs.find(r.db_id);
        if (di == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id " + std::to_string(r.db_id));
        int nl, nr;
        TRY(check_client_for(c, ci->second, di->second, &nl, &nr));
        Shape s = shape_of(c, di->second.L.nu1, di->second.L.nu2);
        need.nu1 = std::max(need.nu1, s.nu1);
        need.nu2 = std::max(need.nu2, s.nu2);
        need.g = std::max(need.g, s.g);
    }
    TRY(ensure_slots(c, L, need, n));
    order.resize(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reqs[a].db_id < reqs[b].db_id; });
    db_of_slot.resize(n);
    for (int k = 0; k < n; k++) {
        sp_request &r = reqs[order[k]];
        Slot &sl = L.slots[k];
        Client &cl = c->clients[r.client_id];
        cl.stamp = ++c->clock;
        fill_desc(c, sl.q, cl, c->dbs[r.db_id]);
        sl.client = r.client_id;
        sl.db = r.db_id;
        L.h_qd[k] = sl.q;
        // the run writes this query's response straight into the pinned staging
        L.h_qd[k].resp = L.h_resp + (uint64_t)k * response_bytes(c->sp);
        db_of_slot[k] = r.db_id;
        // into the lane's pinned staging; the pipeline uploads it
        memcpy(L.h_query + (uint64_t)k * 4 * D, r.query, 4ull * D * 8);
    }
    return SP_OK;
}

int sp_answer_batch(sp_ctx *c, int32_t count, sp_request *reqs) {
    if (!c || !reqs) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_answer_batch");
    Lane &L = c->main;
    std::vector<int> order, dbs;
    int rc = prepare(c, L, count, reqs, order, dbs);
    if (!rc) rc = run_pipeline(c, L, count, dbs, true);
    const uint64_t rb = response_bytes(c->sp);
    // one synchronisation: the pipeline ends with the copies of the responses
    // and of the error flag (also after a failure, so that nothing still
    // reads the staging buffers)
    const cudaError_t se = cudaStreamSynchronize(L.st);
    if (!rc && se != cudaSuccess) rc = fail(SP_ERR_CUDA, std::string("answer: ") + cudaGetErrorString(se));
    if (!rc) rc = take_device_err(c, L);
    if (!rc) {
        for (int k = 0; k < count; k++) memcpy(reqs[order[k]].response, L.h_resp + k * rb, rb);
        rc = collect_stats(c, L);
    }
    L.staged = 0;
    for (int i = 0; i < count; i++) reqs[i].status = rc;
    return rc;
}

int sp_answer(sp_ctx *c, int32_t client_id, int32_t db_id, const uint64_t *query, uint8_t *response,
              uint64_t response_len) {
    sp_request r{client_id, db_id, query, response, response_len, 0};
    return sp_answer_batch(c, 1, &r);
}

int sp_stage_query(sp_ctx *c, int32_t slot, int32_t client_id, int32_t db_id, const uint64_t *query) {
    if (!c || !query) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_stage_query");
    if (slot < 0 || slot >= c->main.cap) return fail(SP_ERR_INVALID, "slot out of range");
    auto ci = c->clients.find(client_id);
    auto di = c->dbs.find(db_id);
    if (ci == c->clients.end() || di == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown client or database");
    int nl, nr;
    TRY(check_client_for(c, ci->second, di->second, &nl, &nr));
    Lane &L = c->main;
    TRY(ensure_slots(c, L, shape_of(c, di->second.L.nu1, di->second.L.nu2), slot + 1));
    Slot &sl = L.slots[slot];
    fill_desc(c, sl.q, ci->second, di->second);
    sl.client = client_id;
    sl.db = db_id;
    L.h_qd[slot] = sl.q;
    CU(cudaMemcpyAsync(sl.query64, query, 4ull * D * 8, cudaMemcpyHostToDevice, L.st));
    CU(launch_narrow(sl.query64, sl.query32, 4, false, L.st));   // 2 rows x 2 primes
    CU(cudaMemcpyAsync(L.d_qd + slot, &L.h_qd[slot], sizeof(QDesc), cudaMemcpyHostToDevice, L.st));
    CU(cudaStreamSynchronize(L.st));
    L.staged = std::max(L.staged, slot + 1);
    return SP_OK;
}

int sp_run_staged(sp_ctx *c, int32_t count) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_run_staged");
    Lane &L = c->main;
    if (count < 1 || count > L.staged) return fail(SP_ERR_INVALID, "count exceeds staged queries");
    std::vector<int> dbs(count);
    for (int k = 0; k < count; k++) {
        dbs[k] = L.slots[k].db;
        if (!c->dbs.count(dbs[k]) || !c->clients.count(L.slots[k].client))
            return fail(SP_ERR_NOT_FOUND, "staged query refers to an unloaded database or client");
    }
    for (int k = 1; k < count; k++)
        if (dbs[k] < dbs[k - 1]) return fail(SP_ERR_INVALID, "stage slots in database order");
    TRY(run_pipeline(c, L, count, dbs, false));
    TRY(check_device_err(c, L));
    return collect_stats(c, L);
}

int sp_time_staged(sp_ctx *c, int32_t count, int32_t iters, double *ms_per_run) {
    if (!c || !ms_per_run) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_time_staged");
    Lane &L = c->main;
    if (count < 1 || count > L.staged || iters < 1) return fail(SP_ERR_INVALID, "count/iters out of range");
    std::vector<int> dbs(count);
    for (int k = 0; k < count; k++) dbs[k] = L.slots[k].db;
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    int rc = SP_OK;
    float tot = 0;
    if (cudaEventRecord(a, L.st) != cudaSuccess) rc = fail(SP_ERR_CUDA, "event record failed");
    for (int i = 0; i < iters && !rc; i++) rc = run_pipeline(c, L, count, dbs, false);
    if (!rc && cudaEventRecord(b, L.st) != cudaSuccess) rc = fail(SP_ERR_CUDA, "event record failed");
    if (!rc) rc = check_device_err(c, L);
    if (!rc && cudaEventElapsedTime(&tot, a, b) != cudaSuccess) rc = fail(SP_ERR_CUDA, "event time failed");
    if (!rc) rc = collect_stats(c, L);   // stage split of the last run only
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!rc) *ms_per_run = tot / iters;
    return rc;
}

int sp_fetch_response(sp_ctx *c, int32_t slot, uint8_t *response, uint64_t response_len) {
    if (!c || !response) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_fetch_response");
    Lane &L = c->main;
    if (slot < 0 || slot >= (int)L.slots.size()) return fail(SP_ERR_INVALID, "slot out of range");
    const uint64_t rb = response_bytes(c->sp);
    if (response_len < rb) return fail(SP_ERR_INVALID, "response buffer too small");
    CU(cudaMemcpyAsync(response, L.slots[slot].q.resp, rb, cudaMemcpyDeviceToHost, L.st));
    CU(cudaStreamSynchronize(L.st));
    return SP_OK;
}

int sp_set_db_mul_variant(sp_ctx *c, int32_t variant) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    if (variant < 0 || variant > 3) return fail(SP_ERR_INVALID, "variant must be 0 (auto), 1, 2 or 3");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_set_db_mul_variant");
    c->mul_force = variant;
    return SP_OK;
}

int sp_set_split_schedule(sp_ctx *c, int32_t shift) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    if (shift != SP_SPLIT_AUTO && shift != SP_SPLIT_NONE && (shift < -4 || shift > 4))
        return fail(SP_ERR_INVALID, "split shift must be SP_SPLIT_AUTO, SP_SPLIT_NONE or in [-4, 4]");
    std::lock_guard<std::mutex> lk(c->mu);
    c->split_force = shift;
    return SP_OK;
}

int sp_tuning_report(sp_ctx *c, char *buf, uint64_t len) {
    if (!c || !buf || !len) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    std::string out;
    for (const auto &kv : c->mul_choice)
        out += "multiply db " + std::to_string(kv.first.first) + " batch class 2^" + std::to_string(kv.first.second) +
               ": variant " + std::to_string(kv.second) + "\n";
    for (const std::string &m : c->tune_log) out += m + "\n";
    const size_t n = std::min<size_t>(out.size(), len - 1);
    std::memcpy(buf, out.data(), n);
    buf[n] = 0;
    return SP_OK;
}

int sp_set_graphs(sp_ctx *c, int32_t on) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_set_graphs");
    c->use_graphs = on != 0;
    return SP_OK;
}

int sp_set_stage_timing(sp_ctx *c, int32_t on) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_set_stage_timing");
    c->stage_timing = on != 0;
    return SP_OK;
}

int sp_stats(sp_ctx *c, sp_stats_out *out) {
    if (!c || !out) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_stats");
    *out = c->stats;
    return SP_OK;
}

int sp_stats_reset(sp_ctx *c) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_stats_reset");
    c->stats = sp_stats_out{};
    return SP_OK;
}

int sp_time_db_mul(sp_ctx *c, int32_t db_id, int32_t nq, int32_t iters, double *ms_per_launch) {
    if (!c || !ms_per_launch) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_time_db_mul");
    Lane &L = c->main;
    auto di = c->dbs.find(db_id);
    if (di == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id");
    if (nq < 1 || nq > L.staged || iters < 1) return fail(SP_ERR_INVALID, "nq/iters out of range");
    for (int k = 0; k < nq; k++)
        if (L.slots[k].db != db_id) return fail(SP_ERR_INVALID, "staged slots must query this database");
    int variant = c->mul_force ? c->mul_force : 1;
    if (!variant_available(c, L, di->second, nq, variant))
        return fail(SP_ERR_UNSUPPORTED, "multiply variant " + std::to_string(variant) +
                                            " is not available for this database and query count");
    CU(cudaEventRecord(L.ev[0], L.st));
    for (int i = 0; i < iters; i++) CU(launch_mul_variant(L, di->second, L.d_qd, nq, variant));
    CU(cudaEventRecord(L.ev[1], L.st));
    TRY(check_device_err(c, L));
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, L.ev[0], L.ev[1]));
    *ms_per_launch = ms / iters;
    return SP_OK;
}

// ---------------------------------------------------------- stage entries
int sp_ntt_fwd(sp_ctx *c, const uint64_t *raw, uint64_t *crt, uint64_t count) {
    if (!c || !raw || !crt || !count) return fail(SP_ERR_INVALID, "NULL argument or zero count");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_ntt_fwd");
    Tmp a(c), b(c);
    TRY(a.get(count * D * 8));
    TRY(b.get(count * 2 * D * 8));
    CU(cudaMemcpyAsync(a.p, raw, count * D * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_to_ntt(a.as<uint64_t>(), b.as<uint32_t>(), (int)count, c->d_tw, c->st));
    Tmp w(c);
    TRY(w.get(count * 2 * D * 8));
    CU(launch_widen(b.as<uint32_t>(), w.as<uint64_t>(), count * 2, false, c->st));
    CU(cudaMemcpyAsync(crt, w.p, count * 2 * D * 8, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_ntt_inv(sp_ctx *c, const uint64_t *crt, uint64_t *raw, uint64_t count) {
    if (!c || !raw || !crt || !count) return fail(SP_ERR_INVALID, "NULL argument or zero count");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_ntt_inv");
    Tmp a(c), n(c), o(c);
    TRY(a.get(count * 2 * D * 8));
    TRY(n.get(count * 2 * D * 4));
    TRY(o.get(count * D * 8));
    CU(cudaMemcpyAsync(a.p, crt, count * 2 * D * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_narrow(a.as<uint64_t>(), n.as<uint32_t>(), count * 2, false, c->st));
    CU(launch_from_ntt(n.as<uint32_t>(), o.as<uint64_t>(), (int)count, c->d_tw, c->st));
    CU(cudaMemcpyAsync(raw, o.p, count * D * 8, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_automorph(sp_ctx *c, const uint64_t *raw, uint64_t *out, uint64_t count, uint32_t t) {
    if (!c || !raw || !out || !count) return fail(SP_ERR_INVALID, "NULL argument or zero count");
    if (!(t & 1)) return fail(SP_ERR_INVALID, "automorphism exponent must be odd");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_automorph");
    Tmp a(c), b(c);
    TRY(a.get(count * D * 8));
    TRY(b.get(count * D * 8));
    CU(cudaMemcpyAsync(a.p, raw, count * D * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_automorph(a.as<uint64_t>(), b.as<uint64_t>(), (int)count, t, c->st));
    CU(cudaMemcpyAsync(out, b.p, count * D * 8, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_expand(sp_ctx *c, int32_t client_id, const uint64_t *query, int32_t nu1, int32_t nu2, int32_t rounds,
              uint64_t *out) {
    if (!c || !query || !out) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_expand");
    auto ci = c->clients.find(client_id);
    if (ci == c->clients.end()) return fail(SP_ERR_NOT_FOUND, "unknown client id");
    if (nu1 < 1 || nu2 < 1 || nu1 > 14 || nu2 > 14) return fail(SP_ERR_INVALID, "nu1/nu2 out of range");
    const Shape s = shape_of(c, nu1, nu2);
    if (s.g > LOGD) return fail(SP_ERR_UNSUPPORTED, "expansion needs more than 11 rounds");
    const int stop = ceil_log2((uint64_t)c->sp.t_gsw * nu2);
    if (rounds <= 0) rounds = s.g;
    if (rounds > s.g) return fail(SP_ERR_INVALID, "rounds exceeds g for this shape");
    const Client &cl = ci->second;
    if (cl.n_left < rounds || cl.n_right < std::min(rounds, stop + 1))
        return fail(SP_ERR_INVALID, "client keys do not cover the requested rounds");
    const uint64_t ct = 4ull * D;
    const uint64_t nout = 1ull << rounds;
    const int max_bits = c->sp.t_gsw * nu2;
    Tmp q64(c), q32(c), v0(c), v1(c), gin(c), qd(c), w(c);
    TRY(q64.get(ct * 8));
    TRY(q32.get(ct * 4));
    TRY(v0.get(ct * 4 * nout));
    TRY(v1.get(ct * 4 * nout));
    TRY(gin.get(ct * 4 * std::max(1, max_bits)));
    TRY(qd.get(sizeof(QDesc)));
    TRY(w.get(ct * 8 * nout));
    QDesc d{};
    d.left = cl.left;
    d.right = cl.right;
    d.query = q32.as<uint32_t>();
    d.v[0] = v0.as<uint32_t>();
    d.v[1] = v1.as<uint32_t>();
    d.gsw_in = gin.as<uint32_t>();
    d.sel = nullptr;
    d.nu1 = nu1;
    d.nu2 = nu2;
    d.g = rounds + 1;            // every executed round writes its outputs
    d.stop = stop;
    d.capture = (stop > 0 && stop < rounds) ? stop : rounds;   // captured only when pruning starts
    d.active = 1;
    CU(cudaMemsetAsync(v0.p, 0, ct * 4 * nout, c->st));
    CU(cudaMemsetAsync(v1.p, 0, ct * 4 * nout, c->st));
    CU(cudaMemcpyAsync(q64.p, query, ct * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_narrow(q64.as<uint64_t>(), q32.as<uint32_t>(), 4, false, c->st));
    CU(cudaMemcpyAsync(qd.p, &d, sizeof(QDesc), cudaMemcpyHostToDevice, c->st));
    for (int r = 0; r < rounds; r++)
        CU(launch_expand_round(qd.as<QDesc>(), 1, r, 2 << r, c->sp, c->d_tw, c->d_neg1, nullptr, c->st));
    uint32_t *fin = (rounds & 1) ? d.v[1] : d.v[0];
    // Entries pruned in the last round(s) are zero; odd entries frozen at
    // stop_round come from the capture buffer.
    if (d.capture < rounds) {
        // clear odd entries of the final buffer, then copy the captured ones in
        for (uint64_t i = 1; i < nout; i += 2)
            CU(cudaMemsetAsync(fin + i * ct, 0, ct * 4, c->st));
        for (int k = 0; k < max_bits && (uint64_t)(2 * k + 1) < nout; k++)
            CU(cudaMemcpyAsync(fin + (2ull * k + 1) * ct, gin.as<uint32_t>() + (uint64_t)k * ct, ct * 4,
                               cudaMemcpyDeviceToDevice, c->st));
    }
    CU(launch_widen(fin, w.as<uint64_t>(), nout * 4, false, c->st));
    CU(cudaMemcpyAsync(out, w.p, ct * 8 * nout, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_regev_to_gsw(sp_ctx *c, int32_t client_id, const uint64_t *regev, int32_t nu2, uint64_t *gsw) {
    if (!c || !regev || !gsw) return fail(SP_ERR_INVALID, "NULL argument");
    if (nu2 < 1 || nu2 > 14) return fail(SP_ERR_INVALID, "nu2 out of range");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_regev_to_gsw");
    auto ci = c->clients.find(client_id);
    if (ci == c->clients.end()) return fail(SP_ERR_NOT_FOUND, "unknown client id");
    const uint64_t ct = 4ull * D;
    const int nin = nu2 * c->sp.t_gsw;
    const uint64_t gwords = (uint64_t)nu2 * 2 * 2 * c->sp.t_gsw * 2 * D;
    Tmp a(c), b(c), g(c), w(c), qd(c);
    TRY(a.get(ct * 8 * nin));
    TRY(b.get(ct * 4 * nin));
    TRY(g.get(gwords * 4));
    TRY(w.get(gwords * 8));
    TRY(qd.get(sizeof(QDesc)));
    QDesc d{};
    d.conv = ci->second.conv;
    d.gsw_in = b.as<uint32_t>();
    d.gsw = g.as<uint32_t>();
    d.nu2 = nu2;
    d.active = 1;
    CU(cudaMemcpyAsync(a.p, regev, ct * 8 * nin, cudaMemcpyHostToDevice, c->st));
    CU(launch_narrow(a.as<uint64_t>(), b.as<uint32_t>(), (uint64_t)nin * 4, false, c->st));
    CU(cudaMemcpyAsync(qd.p, &d, sizeof(QDesc), cudaMemcpyHostToDevice, c->st));
    CU(launch_regev_to_gsw(qd.as<QDesc>(), 1, nin, c->sp, c->d_tw, c->st));
    CU(launch_widen(g.as<uint32_t>(), w.as<uint64_t>(), gwords / D, true, c->st));
    CU(cudaMemcpyAsync(gsw, w.p, gwords * 8, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_gsw_neg(sp_ctx *c, const uint64_t *gsw, int32_t count, uint64_t *neg) {
    if (!c || !gsw || !neg || count < 1) return fail(SP_ERR_INVALID, "NULL argument or bad count");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_gsw_neg");
    const uint64_t words = (uint64_t)count * 2 * 2 * c->sp.t_gsw * 2 * D;
    Tmp a(c), b(c), o(c);
    TRY(a.get(words * 8));
    TRY(b.get(words * 4));
    TRY(o.get(words * 4));
    CU(cudaMemcpyAsync(a.p, gsw, words * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_narrow(a.as<uint64_t>(), b.as<uint32_t>(), words / D, false, c->st));
    CU(launch_gsw_neg(b.as<uint32_t>(), o.as<uint32_t>(), count, c->sp.t_gsw, c->st));
    CU(launch_widen(o.as<uint32_t>(), a.as<uint64_t>(), words / D, false, c->st));
    CU(cudaMemcpyAsync(neg, a.p, words * 8, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_db_mul(sp_ctx *c, int32_t db_id, const uint64_t *sel, uint64_t *acc) {
    if (!c || !sel || !acc) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_mul");
    auto di = c->dbs.find(db_id);
    if (di == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id");
    const DbLayout &L = di->second.L;
    const uint64_t sel_words = (uint64_t)L.rows * 4 * D;
    const uint64_t acc_words = (uint64_t)L.T * L.cols * 4 * D;
    Tmp a(c), s(c), o(c), w(c), qd(c);
    TRY(a.get(sel_words * 8));
    TRY(s.get(sel_words * 4));
    TRY(o.get(acc_words * 4));
    TRY(w.get(acc_words * 8));
    TRY(qd.get(sizeof(QDesc)));
    QDesc d{};
    d.sel = s.as<uint32_t>();
    d.acc = o.as<uint32_t>();
    d.nu1 = L.nu1;
    d.nu2 = L.nu2;
    d.active = 1;
    CU(cudaMemcpyAsync(a.p, sel, sel_words * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_sel_import(a.as<uint64_t>(), s.as<uint32_t>(), L.rows, c->st));
    CU(cudaMemcpyAsync(qd.p, &d, sizeof(QDesc), cudaMemcpyHostToDevice, c->st));
    CU(launch_db_mul(di->second.d, L, qd.as<QDesc>(), 1, c->d_err, c->st));
    CU(launch_widen(o.as<uint32_t>(), w.as<uint64_t>(), acc_words / D, false, c->st));
    CU(cudaMemcpyAsync(acc, w.p, acc_words * 8, cudaMemcpyDeviceToHost, c->st));
    TRY(check_device_err(c, c->main));
    return SP_OK;
}

int sp_db_mul_batch(sp_ctx *c, int32_t db_id, int32_t nq, const uint64_t *sel, uint64_t *acc) {
    if (!c || !sel || !acc) return fail(SP_ERR_INVALID, "NULL argument");
    if (nq < 1 || nq > 1024) return fail(SP_ERR_INVALID, "nq must be in [1, 1024]");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_db_mul_batch");
    auto di = c->dbs.find(db_id);
    if (di == c->dbs.end()) return fail(SP_ERR_NOT_FOUND, "unknown database id");
    const Db &db = di->second;
    const DbLayout &L = db.L;
    const uint64_t sel_words = (uint64_t)L.rows * 4 * D;
    const uint64_t acc_words = (uint64_t)L.T * L.cols * 4 * D;
    Tmp a(c), s(c), o(c), w(c), qd(c);
    TRY(a.get(sel_words * 8));
    TRY(s.get(sel_words * 4 * nq));
    TRY(o.get(acc_words * 4 * nq));
    TRY(w.get(acc_words * 8));
    TRY(qd.get(sizeof(QDesc) * nq));
    std::vector<QDesc> d(nq);
    for (int q = 0; q < nq; q++) {
        d[q] = QDesc{};
        d[q].sel = s.as<uint32_t>() + sel_words * q;
        d[q].acc = o.as<uint32_t>() + acc_words * q;
        d[q].nu1 = L.nu1;
        d[q].nu2 = L.nu2;
        d[q].active = 1;
        CU(cudaMemcpyAsync(a.p, sel + sel_words * q, sel_words * 8, cudaMemcpyHostToDevice, c->st));
        CU(launch_sel_import(a.as<uint64_t>(), d[q].sel, L.rows, c->st));
    }
    CU(cudaMemcpyAsync(qd.p, d.data(), sizeof(QDesc) * nq, cudaMemcpyHostToDevice, c->st));
    int variant = 1;
    TRY(choose_mul_variant(c, c->main, db_id, db, qd.as<QDesc>(), nq, &variant));
    CU(launch_mul_variant(c->main, db, qd.as<QDesc>(), nq, variant));
    for (int q = 0; q < nq; q++) {
        CU(launch_widen(d[q].acc, w.as<uint64_t>(), acc_words / D, false, c->st));
        CU(cudaMemcpyAsync(acc + acc_words * q, w.p, acc_words * 8, cudaMemcpyDeviceToHost, c->st));
        CU(cudaStreamSynchronize(c->st));
    }
    TRY(check_device_err(c, c->main));
    c->stats.db_mul_by_variant[variant - 1]++;
    return SP_OK;
}

int sp_fold(sp_ctx *c, const uint64_t *cts, const uint64_t *gsw, int32_t T, int32_t nu2, uint64_t *out) {
    if (!c || !cts || !gsw || !out) return fail(SP_ERR_INVALID, "NULL argument");
    if (T < 1 || T > c->sp.T || nu2 < 1 || nu2 > 14) return fail(SP_ERR_INVALID, "T or nu2 out of range");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_fold");
    const uint64_t raw_words = ((uint64_t)T * 2 * D) << nu2;
    const uint64_t gwords = (uint64_t)nu2 * 2 * 2 * c->sp.t_gsw * 2 * D;
    Tmp r(c), g64(c), g(c), qd(c);
    TRY(r.get(raw_words * 8));
    TRY(g64.get(gwords * 8));
    TRY(g.get(gwords * 4));
    TRY(qd.get(sizeof(QDesc)));
    QDesc d{};
    d.raw = r.as<uint64_t>();
    d.gsw = g.as<uint32_t>();
    d.nu2 = nu2;
    d.active = 1;
    StageParams sp = c->sp;
    sp.T = T;
    CU(cudaMemcpyAsync(r.p, cts, raw_words * 8, cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(g64.p, gsw, gwords * 8, cudaMemcpyHostToDevice, c->st));
    CU(launch_narrow(g64.as<uint64_t>(), g.as<uint32_t>(), gwords / D, true, c->st));
    CU(cudaMemcpyAsync(qd.p, &d, sizeof(QDesc), cudaMemcpyHostToDevice, c->st));
    for (int lvl = 0; lvl < nu2; lvl++)
        CU(launch_fold_level(qd.as<QDesc>(), 1, lvl, T << (nu2 - 1 - lvl), sp, c->d_tw, nullptr, c->st));
    for (int t = 0; t < T; t++)
        CU(cudaMemcpyAsync(out + (uint64_t)t * 2 * D, r.as<uint64_t>() + ((uint64_t)t << nu2) * 2 * D, 2ull * D * 8,
                           cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

int sp_pack(sp_ctx *c, int32_t client_id, const uint64_t *cts, uint8_t *response, uint64_t response_len) {
    if (!c || !cts || !response) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_pack");
    auto ci = c->clients.find(client_id);
    if (ci == c->clients.end()) return fail(SP_ERR_NOT_FOUND, "unknown client id");
    const uint64_t rb = response_bytes(c->sp);
    if (response_len < rb) return fail(SP_ERR_INVALID, "response buffer too small");
    const int T = c->sp.T;
    Tmp r(c), resp(c), qd(c);
    TRY(r.get((uint64_t)T * 2 * D * 8));
    TRY(resp.get(rb));
    TRY(qd.get(sizeof(QDesc)));
    QDesc d{};
    d.pack = ci->second.pack;
    d.raw = r.as<uint64_t>();
    d.resp = resp.as<uint8_t>();
    d.nu2 = 0;   // one ciphertext per instance
    d.active = 1;
    CU(cudaMemcpyAsync(r.p, cts, (uint64_t)T * 2 * D * 8, cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(qd.p, &d, sizeof(QDesc), cudaMemcpyHostToDevice, c->st));
    CU(launch_pack(qd.as<QDesc>(), 1, c->sp, c->d_tw, nullptr, c->st));
    CU(cudaMemcpyAsync(response, resp.p, rb, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    return verify_guards(c);
}

}  // extern "C"

// ------------------------------------------------------ internal accessors
namespace sp {

int ctx_view(sp_ctx *c, CtxView *out) {
    if (!c || !out) return fail(SP_ERR_INVALID, "NULL argument");
    out->st = c->st;
    out->tw = c->d_tw;
    out->params = c->sp;
    out->mu = &c->mu;
    out->device = c->device;
    out->checked = c->checked;
    return SP_OK;
}

int set_last_error(int code, const char *msg) { return fail(code, msg); }

}  // namespace sp

// ======================================================== serving loop
// Continuous batching: sp_submit queues a request (the query is copied); a
// worker thread launches the queued requests, up to max_batch at a time, on
// whichever lane is free, so a batch admitted while others run overlaps
// with them on the GPU.  When more requests wait than a batch holds, a
// batch gathers the oldest request's database's requests.  Lanes own their
// slots (device workspace sized under the HBM budget), their stream and
// pinned response staging; a finished lane's responses are copied to the
// callers' buffers and their tickets completed.
namespace {

void complete(sp_ctx *c, uint64_t ticket, int status) {
    auto it = c->tickets.find(ticket);
    if (it != c->tickets.end()) {
        it->second.done = 1;
        it->second.status = status;
        it->second.completed = std::chrono::steady_clock::now();
    }
}

void finish_lane(sp_ctx *c, Lane &L) {
    int status = take_device_err(c, L);   // copied by the pipeline before `done`
    if (!status) status = collect_stats(c, L);
    const uint64_t rb = response_bytes(c->sp);
    for (size_t k = 0; k < L.tickets.size(); k++) {
        auto it = c->tickets.find(L.tickets[k]);
        if (it == c->tickets.end()) continue;
        if (!status) memcpy(it->second.response, L.h_resp + k * rb, rb);
        complete(c, L.tickets[k], status);
    }
    c->served += L.tickets.size();
    L.tickets.clear();
    L.busy = false;
    L.staged = 0;
}

// Launch up to L.cap queued requests on lane L (lock held).
void launch_lane(sp_ctx *c, Lane &L) {
    TraceRange trace_("serve_batch");
    std::vector<Pending> batch;
    // batch policy (plan.h batch_rule): the whole queue in arrival order
    // when it fits, else the oldest request's database first
    const BatchRule rule = batch_rule(c->queue.size(), L.cap, c->queue.empty() ? 0 : c->queue.front().db_id);
    for (auto qi = c->queue.begin(); qi != c->queue.end() && (int)batch.size() < L.cap;) {
        if (!rule.takes(qi->db_id)) {
            ++qi;
            continue;
        }
        Pending p = std::move(*qi);
        qi = c->queue.erase(qi);
        // requests that cannot run complete at once with their error
        auto ci = c->clients.find(p.client_id);
        auto di = c->dbs.find(p.db_id);
        int nl, nr;
        if (ci == c->clients.end() || di == c->dbs.end()) {
            fail(SP_ERR_NOT_FOUND, "unknown client or database id");
            complete(c, p.ticket, SP_ERR_NOT_FOUND);
            continue;
        }
        if (int rc = check_client_for(c, ci->second, di->second, &nl, &nr)) {
            complete(c, p.ticket, rc);
            continue;
        }
        batch.push_back(std::move(p));
    }
    if (batch.empty()) return;
    std::vector<sp_request> reqs(batch.size());
    for (size_t k = 0; k < batch.size(); k++)
        reqs[k] = sp_request{batch[k].client_id, batch[k].db_id, batch[k].query.data(), batch[k].response,
                             batch[k].response_len, 0};
    std::vector<int> order, dbs;
    int rc = prepare(c, L, (int)reqs.size(), reqs.data(), order, dbs);
    if (!rc) rc = run_pipeline(c, L, (int)reqs.size(), dbs, true);
    if (!rc && cudaEventRecord(L.done, L.st) != cudaSuccess) rc = fail(SP_ERR_CUDA, "event record failed");
    if (rc) {
        cudaStreamSynchronize(L.st);
        for (auto &p : batch) complete(c, p.ticket, rc);
        c->cv.notify_all();
        return;
    }
    L.tickets.clear();
    for (size_t k = 0; k < order.size(); k++) L.tickets.push_back(batch[order[k]].ticket);
    L.busy = true;
    c->batches++;
}

void serve_worker(sp_ctx *c) {
    cudaSetDevice(c->device);
    std::unique_lock<std::mutex> lk(c->mu);
    for (;;) {
        bool any_busy = false;
        for (Lane *L : c->lanes) {
            if (L->busy && cudaEventQuery(L->done) == cudaSuccess) {
                finish_lane(c, *L);
                c->cv.notify_all();
            }
            any_busy |= L->busy;
        }
        if (!c->queue.empty()) {
            Lane *free_lane = nullptr;
            for (Lane *L : c->lanes)
                if (!L->busy) { free_lane = L; break; }
            if (free_lane) {
                launch_lane(c, *free_lane);
                continue;
            }
        }
        if (c->stopping && c->queue.empty() && !any_busy) break;
        if (any_busy)
            c->cv.wait_for(lk, std::chrono::microseconds(50));
        else
            c->cv.wait(lk, [&] { return c->stopping || !c->queue.empty(); });
    }
}

}  // namespace

extern "C" {

int sp_serve_start(sp_ctx *c, int32_t lanes) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    if (lanes < 1 || lanes > 8) return fail(SP_ERR_INVALID, "lanes must be in [1, 8]");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_serve_start");
    if (c->serving) return fail(SP_ERR_INVALID, "already serving");
    // every lane reserves max_batch workspace slots for the largest loaded
    // database shape now, so admission later only depends on the HBM budget
    // left for client keys
    Shape need{};
    for (auto &kv : c->dbs) {
        Shape s = shape_of(c, kv.second.L.nu1, kv.second.L.nu2);
        need.nu1 = std::max(need.nu1, s.nu1);
        need.nu2 = std::max(need.nu2, s.nu2);
        need.g = std::max(need.g, s.g);
    }
    for (int i = 0; i < lanes; i++) {
        Lane *L = new Lane();
        int rc = lane_init(c, *L, c->p.max_batch);
        if (!rc && need.g) rc = ensure_slots(c, *L, need, c->p.max_batch);
        // then, where the budget allows, the tensor-core multiply workspace
        // for every database that can use it (best effort: without it the
        // lane uses the integer multiplies)
        if (!rc && c->p.max_batch >= 2)
            for (auto &kv : c->dbs)
                if (db_mul_tc_supported(kv.second.L)) ensure_limbs(c, *L, kv.second.L);
        c->lanes.push_back(L);
        if (rc) {
            for (Lane *x : c->lanes) {
                lane_free(c, *x);
                delete x;
            }
            c->lanes.clear();
            return rc;
        }
    }
    c->serving = true;
    c->stopping = false;
    c->worker = std::thread(serve_worker, c);
    return SP_OK;
}

int sp_serve_stop(sp_ctx *c) {
    if (!c) return fail(SP_ERR_INVALID, "NULL context");
    {
        std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_serve_stop");
        if (!c->serving) return SP_OK;
        c->stopping = true;
    }
    c->cv.notify_all();
    if (c->worker.joinable()) c->worker.join();
    std::lock_guard<std::mutex> lk(c->mu);
    for (Lane *L : c->lanes) {
        lane_free(c, *L);
        delete L;
    }
    c->lanes.clear();
    c->serving = false;
    c->stopping = false;
    return SP_OK;
}

int sp_submit(sp_ctx *c, const sp_request *req, uint64_t *ticket) {
    if (!c || !req || !ticket || !req->query || !req->response) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_submit");
    if (!c->serving || c->stopping) return fail(SP_ERR_INVALID, "serving loop not running (sp_serve_start)");
    if (req->response_len < response_bytes(c->sp)) return fail(SP_ERR_INVALID, "response buffer too small");
    Pending p;
    p.ticket = c->next_ticket++;
    p.client_id = req->client_id;
    p.db_id = req->db_id;
    p.query.assign(req->query, req->query + 4ull * D);
    p.response = req->response;
    p.response_len = req->response_len;
    TicketState ts;
    ts.response = req->response;
    ts.submitted = std::chrono::steady_clock::now();
    c->tickets[p.ticket] = ts;
    *ticket = p.ticket;
    c->queue.push_back(std::move(p));
    c->cv.notify_all();
    return SP_OK;
}

int sp_poll(sp_ctx *c, uint64_t ticket, int32_t *done, int32_t *status) {
    if (!c || !done || !status) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_poll");
    auto it = c->tickets.find(ticket);
    if (it == c->tickets.end()) return fail(SP_ERR_NOT_FOUND, "unknown ticket");
    *done = it->second.done;
    *status = it->second.status;
    if (it->second.done) c->tickets.erase(it);
    return SP_OK;
}

int sp_wait(sp_ctx *c, uint64_t ticket, int32_t *status) {
    double ms = 0;
    return sp_wait_timed(c, ticket, status, &ms);
}

int sp_wait_timed(sp_ctx *c, uint64_t ticket, int32_t *status, double *server_ms) {
    if (!c || !status || !server_ms) return fail(SP_ERR_INVALID, "NULL argument");
    std::unique_lock<std::mutex> lk(c->mu);
    auto it = c->tickets.find(ticket);
    if (it == c->tickets.end()) return fail(SP_ERR_NOT_FOUND, "unknown ticket");
    c->cv.wait(lk, [&] { return c->tickets[ticket].done != 0; });
    const TicketState &ts = c->tickets[ticket];
    *status = ts.status;
    *server_ms = std::chrono::duration<double, std::milli>(ts.completed - ts.submitted).count();
    c->tickets.erase(ticket);
    return SP_OK;
}

int sp_serve_stats(sp_ctx *c, uint64_t *served, uint64_t *batches, uint64_t *queued) {
    if (!c || !served || !batches || !queued) return fail(SP_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(c->mu);
    TraceRange trace_("sp_serve_stats");
    *served = c->served;
    *batches = c->batches;
    *queued = c->queue.size();
    return SP_OK;
}

}  // extern "C"
