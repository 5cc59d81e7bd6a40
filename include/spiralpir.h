/*
 * spiralpir.h - C ABI of the GB300 Spiral PIR answer path (libspiralpir.so).
 *
 * Drop-in for the server answer path of EricArcherman/GPU-PIR.  The
 * reference has no callable answer API: its host boundary is gpu-pir/host.h
 * (C++ linkage, std::string/std::vector arguments, errors call exit) and the
 * answer flow lives in the test main()s (gpu-pir/fold_test.cu:30-94,
 * gpu-pir/db_mul_test.cu:62-212, gpu-pir/expansion_test.cu:33-113).  Each
 * entry point below names the reference code it replaces.
 *
 * Conventions
 *  - Every function returns SP_OK (0) or an SP_ERR_* code and never exits
 *    the process; sp_last_error() returns the calling thread's message.
 *  - All buffers are host buffers owned by the caller; calls copy in and out.
 *  - Polynomials use the layouts of the reference's golden vectors
 *    (gpu-pir/test_data, written by spiral-rs): D = 2048 coefficients;
 *      raw poly   uint64[D]          coefficients mod q = q1*q2
 *      CRT poly   uint64[2][D]       NTT form mod q1 then mod q2, values < q_i
 *      ciphertext [2 rows][...]      Regev ciphertext rows (-a, s*a+e+m)
 *      matrix     [rows][cols][...]  row-major
 *  - q1 = 268369921, q2 = 249561089 (gpu-pir/params.cuh:25-31).
 *  - A context is internally locked; calls from several threads serialise.
 */
#ifndef SPIRALPIR_H
#define SPIRALPIR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SP_OK 0
#define SP_ERR_INVALID 1     /* bad argument, size or shape */
#define SP_ERR_CUDA 2        /* CUDA runtime error */
#define SP_ERR_NOMEM 3       /* device allocation failed or HBM budget exceeded */
#define SP_ERR_NOT_FOUND 4   /* unknown database or client id */
#define SP_ERR_DEVICE 5      /* a device-side check failed (bounded wait ran out) */
#define SP_ERR_UNSUPPORTED 6 /* parameter combination not implemented */
#define SP_ERR_IO 7          /* a file could not be opened, read or written */

#define SP_D 2048

typedef struct sp_ctx sp_ctx;

/* Ring/gadget parameters shared by every database and client of a context.
 * Replaces the compile-time constants of gpu-pir/params.cuh:49-71. */
typedef struct sp_params {
    int32_t n;           /* plaintext matrices are n x n (1, 2 or 4) */
    int32_t pt_bits;     /* plaintext modulus p = 2^pt_bits (<= 8) */
    int32_t t_exp_left;  /* expansion gadget length, first-dimension branch */
    int32_t t_exp_right; /* expansion gadget length, GSW-bit branch */
    int32_t t_gsw;       /* GSW / folding gadget length */
    int32_t t_conv;      /* Regev->GSW conversion and packing gadget length */
    int32_t q2_bits;     /* response first row is switched to 2^q2_bits */
    int32_t max_batch;   /* queries answered concurrently (workspace slots) */
} sp_params;

/* Per-stage device time accumulated since the last sp_stats_reset (the
 * stage fields only for runs with stage timing on: sp_set_stage_timing). */
typedef struct sp_stats_out {
    uint64_t answers;        /* queries answered */
    uint64_t launches;       /* kernel launches issued by answers */
    double ms_expand;        /* coefficient expansion */
    double ms_convert;       /* Regev->GSW conversion past the expansion (join) */
    double ms_db_mul;        /* first-dimension multiply */
    double ms_fold;          /* DB output to raw + folding */
    double ms_pack;          /* packing, modulus switch, serialisation */
    double ms_total;         /* device time of whole answers */
    uint64_t db_mul_calls;   /* first-dimension multiply launches */
    uint64_t db_mul_bytes;   /* algorithmic bytes of those launches */
    uint64_t db_mul_by_variant[3]; /* multiplies run by variant 1, 2, 3 */
} sp_stats_out;

/* One request of a batch. */
typedef struct sp_request {
    int32_t client_id;
    int32_t db_id;
    const uint64_t *query;   /* NTT ciphertext uint64[2][2][D] */
    uint8_t *response;       /* sp_response_bytes() bytes */
    uint64_t response_len;
    int32_t status;          /* out: SP_OK or an error code */
} sp_request;

/* ------------------------------------------------------------------ */
/* Context (replaces gen_twiddles_gpu / checkLast, gpu-pir/host.cu:79-138) */
int sp_ctx_create(const sp_params *params, uint64_t hbm_budget_bytes, sp_ctx **out);
int sp_ctx_destroy(sp_ctx *ctx);
int sp_last_error(char *buf, size_t len);
int sp_response_bytes(const sp_ctx *ctx, uint64_t *bytes);
int sp_hbm_used(const sp_ctx *ctx, uint64_t *bytes);
/* Checked mode (environment variable SPIRALPIR_CHECKED=1 when the context is
 * created; no counterpart in the reference): every device allocation, and
 * every buffer carved out of a query slot, is followed by a guard region of
 * fill bytes, checked after each synchronous call, so that a kernel writing
 * past the end of a buffer is reported as SP_ERR_DEVICE naming the buffer.
 * Context creation verifies that the check catches one flipped guard byte.
 * sp_check_guards sets *checked (1 in checked mode) and verifies the guards
 * now (SP_OK when checked mode is off). */
int sp_check_guards(sp_ctx *ctx, int32_t *checked);
/* Failure-path self-test of the device waits (no counterpart in the
 * reference): runs one kernel whose barrier wait nothing completes, with the
 * multiply kernels' bounded wait shortened to limit_ms (1 .. 1000).  The
 * wait gives up, the kernel sets the device error flag and returns, and the
 * call returns SP_ERR_DEVICE; the context stays usable.  No GPU fault. */
int sp_wait_probe(sp_ctx *ctx, int32_t limit_ms);

/* ------------------------------------------------------------------ */
/* Databases.  Record i = row * 2^nu2 + col; a record is n*n plaintext
 * polynomials of D coefficients in [0, p), one byte each. */

/* Encode plaintext records into the device CRT-NTT image (the encoder the
 * reference leaves as a note, gpu-pir/optplan.md:80-84). */
int sp_db_load_plain(sp_ctx *ctx, int32_t db_id, const uint8_t *records, uint64_t n_records,
                     int32_t nu1, int32_t nu2);
/* Load an image already in NTT form: uint32 planes [n*n][2^nu2][2^nu1][2][D]
 * (the reference's Database<Poly<uint32_t>> layout col[c].row[r].crt[k],
 * gpu-pir/structures.cuh:200-210, load_db gpu-pir/db_mul_test.cu:23-34). */
int sp_db_load_ntt(sp_ctx *ctx, int32_t db_id, const uint32_t *planes, int32_t nu1, int32_t nu2);
int sp_db_unload(sp_ctx *ctx, int32_t db_id);
/* Checkpoint of an encoded database image (no counterpart in the reference,
 * which has no encoder).  sp_db_save writes a 64-byte header (magic
 * "SPIRDB1", version, layout (2: 28-bit residues, 8 per 7 words), n, pt_bits,
 * nu1, nu2, d, q1, q2, image bytes, FNV-1a-64 over the image's 64-bit words)
 * followed by the device image;
 * sp_db_restore loads
 * such a file as database `db_id`, skipping the encode.  The file must match
 * the context's n and pt_bits; a short file or a checksum mismatch gives
 * SP_ERR_INVALID and loads nothing, file errors SP_ERR_IO. */
int sp_db_save(sp_ctx *ctx, int32_t db_id, const char *path);
int sp_db_restore(sp_ctx *ctx, int32_t db_id, const char *path);

/* ------------------------------------------------------------------ */
/* Client public parameters, uint64 CRT form (load_polys(.., crt_form, montgomery)
 * gpu-pir/host.cu:216-249; PublicParameters gpu-pir/structures.cuh:173-177):
 *   exp_left  [n_left][2][t_exp_left][2][D]
 *   exp_right [n_right][2][t_exp_right][2][D]
 *   conv      [2][2*t_conv][2][D]
 *   pack      [n][n+1][t_conv][2][D]                                  */
int sp_client_set_keys(sp_ctx *ctx, int32_t client_id, const uint64_t *exp_left, int32_t n_left,
                       const uint64_t *exp_right, int32_t n_right, const uint64_t *conv,
                       const uint64_t *pack);
/* The same keys with their uniform rows given by a 32-byte seed (the
 * "public parameters: store the RNG seed as sent, expand the RNG on the GPU"
 * plan of gpu-pir/optplan.md:88-92): row 0 of every key matrix is
 * regenerated on the device from `seed` (ChaCha20 block function of
 * RFC 8439: key = seed, counter = block, nonce = (row-0 polynomial index,
 * prime index, 0x3153504B); block b gives residues 8b..8b+7, each the 64-bit
 * word of two consecutive block words reduced mod the prime; polynomials are
 * numbered left (matrix, column), right, conversion (column), packing
 * (matrix, column)).  The other rows are passed, uint64 CRT form:
 *   left_rest  [n_left][t_exp_left][2][D]     (row 1)
 *   right_rest [n_right][t_exp_right][2][D]   (row 1)
 *   conv_rest  [2*t_conv][2][D]               (row 1)
 *   pack_rest  [n][n][t_conv][2][D]           (rows 1..n)
 * The upload shrinks by one row of each matrix (about half). */
int sp_client_set_keys_seeded(sp_ctx *ctx, int32_t client_id, const uint8_t *seed, const uint64_t *left_rest,
                              int32_t n_left, const uint64_t *right_rest, int32_t n_right, const uint64_t *conv_rest,
                              const uint64_t *pack_rest);
int sp_client_evict(sp_ctx *ctx, int32_t client_id);

/* ------------------------------------------------------------------ */
/* Answering (the flow of the reference's test main()s, wired end to end):
 * expansion -> Regev->GSW -> G - C -> first-dimension multiply -> fold ->
 * pack -> modulus switch -> serialise. */
int sp_answer(sp_ctx *ctx, int32_t client_id, int32_t db_id, const uint64_t *query,
              uint8_t *response, uint64_t response_len);
int sp_answer_batch(sp_ctx *ctx, int32_t count, sp_request *reqs);

/* Device-resident answering for throughput measurement: stage queries into
 * workspace slots (host->device), run the answer on resident data, fetch
 * responses (device->host) separately.  sp_answer / sp_answer_batch use the
 * same slots and consume any staged queries. */
int sp_stage_query(sp_ctx *ctx, int32_t slot, int32_t client_id, int32_t db_id, const uint64_t *query);
int sp_run_staged(sp_ctx *ctx, int32_t count);
int sp_fetch_response(sp_ctx *ctx, int32_t slot, uint8_t *response, uint64_t response_len);
/* Run the staged queries `iters` times back to back on the context's stream,
 * timed with CUDA events on that stream; ms per run of all `count` queries. */
int sp_time_staged(sp_ctx *ctx, int32_t count, int32_t iters, double *ms_per_run);

/* First-dimension multiply variant for launches with several queries on one
 * database: 0 = autotune (default: per database and size class ceil(log2 nq),
 * the best batched candidate is timed once against nq times the per-query
 * kernel's one-query time, and the faster is kept), 1 = per-query streaming
 * kernel (TMA-fed, HBM-bound), 2 = batched integer kernel (each residue read
 * once per 8 queries), 3 = tensor-core kernel (exact fp16 digit products, up
 * to 32 queries per pass over the image; needs 128 combos per block and at
 * most 512 rows, and a workspace of rows * 2 MiB + up to 512 MiB per pipeline
 * lane).  A forced variant that does not apply falls back to the autotuner.
 * sp_time_db_mul times the forced variant (1 when none is forced).  The
 * result is identical. */
int sp_set_db_mul_variant(sp_ctx *ctx, int32_t variant);
/* Answer pipelines run as CUDA graphs (default on): the launches of a batch
 * plan (query count, expansion and fold depths, and the database, length and
 * multiply variant of each run of slots) are captured once per pipeline lane
 * and replayed.  Off: the same launches are issued one by one.  Reloading a
 * database drops the captured graphs.  No counterpart in the reference. */
int sp_set_graphs(sp_ctx *ctx, int32_t on);
/* Per-stage device time in sp_stats (default off).  On: each answer run
 * records an event between every two stages (expansion, conversion join,
 * multiply, output to raw + folds, pack), about 5 us each, and sp_stats
 * accumulates ms_expand .. ms_pack.  Off: those fields stay 0, ms_total is
 * still measured, and each stage's first kernel starts as a dependent launch
 * of the previous stage's last.  The responses are identical.  No
 * counterpart in the reference. */
int sp_set_stage_timing(sp_ctx *ctx, int32_t on);
/* Serving loop (continuous batching).  sp_serve_start starts a worker thread
 * with `lanes` pipeline lanes (each its own stream and max_batch workspace
 * slots).  sp_submit copies the request's query and returns a ticket; the
 * worker coalesces queued requests into batches of up to max_batch and
 * launches each on a free lane, so batches admitted while others run overlap
 * on the GPU.  The response is written to the request's buffer before the
 * ticket completes (sp_poll / sp_wait); a request that cannot run (unknown
 * ids, keys that do not cover the database, workspace beyond the HBM
 * budget) completes with its error status.  sp_serve_start reserves each
 * lane's workspace for the largest database loaded at that time.
 * sp_serve_stop drains the queue. */
int sp_serve_start(sp_ctx *ctx, int32_t lanes);
int sp_serve_stop(sp_ctx *ctx);
int sp_submit(sp_ctx *ctx, const sp_request *req, uint64_t *ticket);
int sp_poll(sp_ctx *ctx, uint64_t ticket, int32_t *done, int32_t *status);
int sp_wait(sp_ctx *ctx, uint64_t ticket, int32_t *status);
/* sp_wait that also returns the request's server-side latency: milliseconds
 * from sp_submit to the response bytes being written (steady clock). */
int sp_wait_timed(sp_ctx *ctx, uint64_t ticket, int32_t *status, double *server_ms);
int sp_serve_stats(sp_ctx *ctx, uint64_t *served, uint64_t *batches, uint64_t *queued);

/* Split schedule of the narrow launches (no counterpart in the reference):
 * an expansion round, fold level or pack with few items spreads each item
 * over split = min(SMs / items, cap) CTAs, shifted by the schedule (shift
 * s: x 2^s, s < 0: / 2^-s; SP_SPLIT_NONE: one CTA per item).  By default
 * (SP_SPLIT_AUTO) the schedule is autotuned per batch class (ceil(log2 of
 * the query count), deepest expansion, deepest fold): on a class's first run
 * the pipeline runs once untimed, then once per candidate (0, -1, +1, none)
 * on the batch at hand, and the fastest is kept.  Results are identical under every
 * schedule.  sp_tuning_report writes the multiply-variant choices and the
 * tuned classes (candidate times, choice) as text lines into buf. */
#define SP_SPLIT_AUTO 127
#define SP_SPLIT_NONE (-16)
int sp_set_split_schedule(sp_ctx *ctx, int32_t shift);
int sp_tuning_report(sp_ctx *ctx, char *buf, uint64_t len);
int sp_stats(sp_ctx *ctx, sp_stats_out *out);
int sp_stats_reset(sp_ctx *ctx);
/* Time `iters` launches of the first-dimension multiply of db_id on the
 * selectors staged in slots [0, nq) with CUDA events; ms per launch. */
int sp_time_db_mul(sp_ctx *ctx, int32_t db_id, int32_t nq, int32_t iters, double *ms_per_launch);

/* ------------------------------------------------------------------ */
/* Stage entry points on host buffers, for parity tests.                */

/* raw -> CRT NTT form (NTT_R, gpu-pir/ntt_28bit.cuh:251-270). */
int sp_ntt_fwd(sp_ctx *ctx, const uint64_t *raw, uint64_t *crt, uint64_t count);
/* CRT NTT form -> raw: INTT + inverse CRT (INTT_R + from_ntt_regs,
 * gpu-pir/ntt_28bit.cuh:292-314, gpu-pir/gadget.cuh:8-24). */
int sp_ntt_inv(sp_ctx *ctx, const uint64_t *crt, uint64_t *raw, uint64_t count);
/* raw x -> x^t (automorph, gpu-pir/automorph.cuh:54-61). */
int sp_automorph(sp_ctx *ctx, const uint64_t *raw, uint64_t *out, uint64_t count, uint32_t t);
/* Coefficient expansion with the client's keys (coefficient_expansion_r,
 * gpu-pir/expansion.cuh:222-259): `rounds` rounds (0 = all g rounds for
 * the shape) of query uint64[2][2][D] into out uint64[2^rounds][2][2][D]. */
int sp_expand(sp_ctx *ctx, int32_t client_id, const uint64_t *query, int32_t nu1, int32_t nu2,
              int32_t rounds, uint64_t *out);
/* Regev -> GSW with the client's conversion key (the slot
 * PublicParameters.conversion, gpu-pir/structures.cuh:176):
 *   regev uint64[nu2*t_gsw][2][2][D] -> gsw uint64[nu2][2][2*t_gsw][2][D] */
int sp_regev_to_gsw(sp_ctx *ctx, int32_t client_id, const uint64_t *regev, int32_t nu2, uint64_t *gsw);
/* G - C for `count` GSW ciphertexts [2][2*t_gsw][2][D] (v_folding_neg). */
int sp_gsw_neg(sp_ctx *ctx, const uint64_t *gsw, int32_t count, uint64_t *neg);
/* First-dimension multiply (db_mul_kernel, gpu-pir/db_mul.cuh:26-70):
 *   sel uint64[2^nu1][2][2][D] -> acc uint64[n*n][2^nu2][2][2][D] */
int sp_db_mul(sp_ctx *ctx, int32_t db_id, const uint64_t *sel, uint64_t *acc);
/* The same multiply for `nq` selector sets in one launch, by the variant
 * that sp_set_db_mul_variant forces (autotuned when none):
 *   sel uint64[nq][2^nu1][2][2][D] -> acc uint64[nq][n*n][2^nu2][2][2][D]
 * No counterpart in the reference (its multiply test runs one query). */
int sp_db_mul_batch(sp_ctx *ctx, int32_t db_id, int32_t nq, const uint64_t *sel, uint64_t *acc);
/* Fold (FOLD_CIPHERTEXTS, gpu-pir/folding.cuh:45-65) of T instances:
 *   cts uint64[T][2^nu2][2][D] raw, gsw uint64[nu2][2][2*t_gsw][2][D]
 *   -> out uint64[T][2][D] raw.  (G - C is derived, not passed.) */
int sp_fold(sp_ctx *ctx, const uint64_t *cts, const uint64_t *gsw, int32_t T, int32_t nu2, uint64_t *out);
/* Fold without allocating device memory: same inputs, output and result as
 * sp_fold, for callers that may not call cudaMalloc at that point (a process
 * whose device memory another allocator already holds, or a service that
 * allocates only at start-up).  No counterpart in the reference.  Device
 * storage is a fixed 8 MiB + 4 KiB array the library declares per GPU, held
 * until the process exits; inputs needing more than 8 MiB (T * 2^nu2 * 32 KiB
 * of ciphertexts plus nu2 * t_gsw * 192 KiB for the GSW ciphertexts, as
 * uploaded and in Montgomery form) are rejected with SP_ERR_INVALID.  The
 * call runs on the context's GPU whatever device the calling thread has
 * current (restored on return).  The first call for a GPU resolves the
 * array's device address there (cudaGetSymbolAddress); make that first call
 * before any stream capture.  All calls share the one array: calls are
 * serialised by a process-wide lock and each waits for its own GPU work,
 * since two calls overlapping on the GPU would race on it.  In checked mode a
 * guard region after the call's data in the array is verified after the
 * fold. */
int sp_fold_noalloc(sp_ctx *ctx, const uint64_t *cts, const uint64_t *gsw, int32_t T, int32_t nu2, uint64_t *out);
/* Pack n*n raw ciphertexts uint64[n*n][2][D] with the client's packing
 * keys, modulus-switch and serialise into `response`. */
int sp_pack(sp_ctx *ctx, int32_t client_id, const uint64_t *cts, uint8_t *response, uint64_t response_len);

#ifdef __cplusplus
}
#endif

#endif /* SPIRALPIR_H */
