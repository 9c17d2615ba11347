/*
 * covgpu.h -- C ABI of libcovgpu.so, the GB300 (sm_103a) covering-code
 * search and verification library.
 *
 * Conventions (kept from the reference's own C-ABI libraries,
 * cov/gemm2/dct.cu:55-57 and cov/gemm2/chainsolve.cu:370-433):
 *   - every entry point returns int: 0 = ok, negative = error;
 *     -(100 + cudaError_t) for a CUDA runtime error;
 *   - host buffers are plain pointers owned by the caller; the library owns
 *     device memory between *_create and *_destroy;
 *   - the library spawns no threads; one caller thread per handle.
 * Codewords are uint8 digits, MSB first: word index x = sum_j w_j q^(n-1-j)
 * (cov/engine/covsearch2e.c:916-921, cov/verify_cov.py:27-35).
 *
 * Domain (the reference engine's own limits, covsearch2e.c:1111-1117, and
 * this library's packing): 2 <= q <= 16, 1 <= n <= 16, 0 <= R,
 * q^n < 2^32, 1 <= M <= 65535.
 */
#ifndef COVGPU_H
#define COVGPU_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COV_OK              0
#define COV_EINVAL         -1   /* bad parameter / outside the domain       */
#define COV_ENOMEM         -2   /* device allocation failed                  */
#define COV_ESTATE         -3   /* call out of order (e.g. run before load)  */
#define COV_ETIMEOUT       -4   /* a bounded device-side wait gave up        */
#define COV_EDRIFT         -5   /* an in-kernel invariant check failed       */
#define COV_ENODEV         -6   /* no usable sm_103 device                   */
#define COV_ERANGE         -7   /* request exceeds a fixed capacity          */

/* One record per tabu move; the oracle writes the same layout, so traces of
 * the two compare byte for byte.  Fields follow the per-iteration steps of
 * cov/engine/covsearch2e.c:1304-1580. */
typedef struct {
    int64_t it;         /* 1-based iteration number (covsearch2e.c:1325)    */
    int64_t u;          /* index of the sampled uncovered word (:1335)      */
    int64_t delta;      /* evaluated delta of the committed move (:1476)    */
    int64_t unc;        /* uncovered count right after the commit (:1528)   */
    int64_t unc_end;    /* uncovered count at the end of the iteration,
                           i.e. after a kick when one happened (:1553-1579) */
    int64_t best;       /* best uncovered count after the iteration         */
    int32_t ncand;      /* candidate moves collected (:1359-1380)           */
    int32_t ncw;        /* distinct candidate codewords (:1458-1465)        */
    int32_t i, p, v;    /* committed move: codeword, position, new value    */
    int32_t kicked;     /* 1 when the iteration ended in a kick; with --sa
                           bit 0 is the stall reheat and bit 1 a rejected
                           proposal (i, p, v, delta are the proposal's)   */
} cov_move_rec;


/* ------------------------------------------------------------------------
 * Search instances.
 *
 * A pool holds up to max_slots independent searches ("slots"); every call
 * to cov_pool_run advances all live slots together in one launch, one
 * thread-block cluster of `cluster` CTAs per slot.  A single covsearch2e
 * process is a pool with one slot and a wide cluster; batched restarts and
 * served requests are pools with many slots.
 *
 * Replaces the process boundary covengine / campaign.py cross today
 * (cov/engine/covengine:624-643, cov/campaign.py:54-86): the arguments are
 * covsearch2e's -q -n -R -M -s --tabu --kick --stall --cand --wide
 * (cov/engine/covsearch2e.c:1042-1095).
 * --------------------------------------------------------------------- */
typedef struct cov_pool cov_pool;

typedef struct {
    int32_t q, n, R, M;
    uint64_t seed;        /* -s       (covsearch2e default 12345)           */
    int32_t tabu;         /* --tabu   tenure (default 0)                    */
    int32_t kick;         /* --kick   codewords moved per kick (default 2)  */
    int32_t cand;         /* --cand   candidate sample cap (default 100000) */
    int32_t trace;        /* 1 = keep a cov_move_rec per move               */
    int64_t stall;        /* --stall  moves without improvement (5000)      */
    int64_t trace_cap;    /* records kept when trace = 1                    */
    int32_t wide;         /* --wide  all n(q-1) moves of a candidate codeword
                           *         (covsearch2e.c:1353-1376); 0 = off     */
    int32_t fix0;         /* --fix0  translate the initial code so codeword 0
                           *         is 0^n and never move it
                           *         (covsearch2e.c:1241-1253, :1343, :1359,
                           *         :1560); 0 = off                        */
    int32_t sa;           /* --sa    focused simulated annealing instead of
                           *         the tabu selection (:1408-1441); 0 = off */
    int32_t noise;        /* --noise per-mille of moves taken unevaluated
                           *         (:1443-1448); 0 = off                  */
    double t0, cool, tmin; /* --t0 --cool --tmin of --sa
                           *         (reference defaults 0.6, 0.999999, 0.02) */
} cov_params;

typedef struct {
    int64_t it;           /* iterations made (RESULT iters=)                */
    int64_t uncovered;    /* current uncovered count                        */
    int64_t best;         /* best uncovered count (RESULT uncovered=)       */
    int64_t kicks;        /* RESULT kicks=                                  */
    int64_t trace_n;      /* moves recorded so far                          */
    int32_t status;       /* 0 or a COV_E* code                             */
    int32_t finished;     /* 1 once the code covers                         */
    int32_t ul_valid;     /* uncovered-word list currently valid            */
    int32_t ul_n;         /* its length (including stale entries)           */
} cov_status;

/* cov/gemm2/chainsolve.cu:370-375 (chain_run) is the reference's batched
 * GPU entry; cov_pool_* generalises it to uneven instances. */
int cov_pool_create(int32_t max_slots, int32_t cluster, cov_pool **out);
int cov_pool_set_budget(cov_pool *pool, double seconds);   /* per-launch wall limit */
/* Tuning knob by name: "neg_cluster_pairs" (list x candidate pairs from
 * which the whole cluster shares the uncovered-list pass), "list_cost"
 * (weight of one uncovered-list entry against one walked word when the
 * entering side chooses between them, covsearch2e.c:1466-1467),
 * "grid_help" (a pool with one slot: up to `value` helper clusters, on the
 * SMs its cluster leaves free, share the commit of each move; 0 = off; the
 * launch then holds the whole GPU and must not share it with other work).
 * None changes a trajectory. */
int cov_pool_set_param(cov_pool *pool, const char *name, int64_t value);
/* Per-slot setting by name: "cluster" (CTAs per instance, 1..16; slots of
 * each cluster size run as one launch, the launches of a step side by side),
 * "neg_cluster_pairs" and "list_cost" (this slot only), "adjust_mode"
 * (private-count upkeep of a commit: 0 per thread, 1 aggregated per warp,
 * -1 chosen from the expected event count), "it_limit" (iteration count at which
 * the slot stops; -1 none), "wide_sliced" (the --wide list pass finds the
 * hits of up to 64 candidates by bit-sliced counts: 1, the default; or tests
 * every pair: 0).  None changes a trajectory.  chain_run (cov/gemm2/chainsolve.cu:370-375)
 * takes one iteration budget for all chains; covengine gives each chain its
 * own time budget (cov/engine/covengine:624-643). */
int cov_pool_set_slot_param(cov_pool *pool, int32_t slot, const char *name, int64_t value);
/* The reference's batched GPU entry with its exact arguments and buffers:
 * chain_run (cov/gemm2/chainsolve.cu:370-375, bound by
 * cov/gemm2/chain.py:30-57).  code_h and best_h hold nchains x M rows of 16
 * digits (digits past n are 0 in best_h); best_u_h, solved_h and iters_h
 * one entry per chain.  Each chain runs the p5b trajectory from its own
 * start code with seed seed*1000003 + chain*7919 for at most `iters` moves;
 * `threads` is accepted and unused.  Returns 0 or a COV_E* code. */
int cov_chain_run(int q, int n, int R, int M, int nchains, long long iters,
                  unsigned long long seed, int threads, const uint8_t *code_h,
                  uint8_t *best_h, int32_t *best_u_h, int32_t *solved_h,
                  long long *iters_h);
/* Free and total bytes of the current device (cudaMemGetInfo), for
 * admitting instances by free HBM.  No counterpart in the reference, whose
 * solvers run as CPU processes. */
int cov_device_memory(int64_t *free_bytes, int64_t *total_bytes);
/* Device bytes one slot with these parameters occupies (0 = invalid). */
size_t cov_slot_bytes(const cov_params *prm);
/* Add an instance and build its initial state from `m` codewords
 * (m*n digits): m == M rebuild, m < M greedy placement (or random digits
 * when random_init), m > M remove-and-repair -- covsearch2e.c:1156-1255. */
int cov_pool_add(cov_pool *pool, const cov_params *prm, const uint8_t *code,
                 int32_t m, int32_t random_init, int32_t *slot);
/* Re-initialise a live slot from a new seed and code (m <= the number of
 * codewords the slot was created for), reusing its device storage. */
int cov_pool_load(cov_pool *pool, int32_t slot, uint64_t seed,
                  const uint8_t *code, int32_t m, int32_t random_init);
/* Advance every live slot by up to `moves` moves; stop a slot early when
 * it covers or when best <= target (target < 0: none).
 * covsearch2e.c:1304-1580. */
int cov_pool_run(cov_pool *pool, int64_t moves, int64_t target);
/* The same, queued on the pool's stream without waiting; cov_pool_sync
 * waits.  cov_pool_graph_run queues `steps` such runs captured once as a
 * CUDA graph (re-captured when moves/target/steps or the slot set change). */
int cov_pool_run_async(cov_pool *pool, int64_t moves, int64_t target);
int cov_pool_graph_run(cov_pool *pool, int64_t moves, int64_t target, int32_t steps);
int cov_pool_sync(cov_pool *pool);
/* Queue the pool's work on the caller's cudaStream_t (passed as void*);
 * NULL returns to the pool's own stream. */
int cov_pool_set_stream(cov_pool *pool, void *stream);
/* Statuses of slots 0..n-1 in one copy (unused slots report COV_ESTATE). */
int cov_pool_status_all(cov_pool *pool, cov_status *out, int32_t n);
int cov_pool_status(cov_pool *pool, int32_t slot, cov_status *out);
int cov_pool_get_code(cov_pool *pool, int32_t slot, uint8_t *out);  /* M*n current */
int cov_pool_get_best(cov_pool *pool, int32_t slot, uint8_t *out);  /* M*n best    */
int cov_pool_get_cnt(cov_pool *pool, int32_t slot, uint16_t *out);  /* q^n counts  */
int cov_pool_get_private(cov_pool *pool, int32_t slot, int32_t *out); /* M*(n+1)   */
int cov_pool_get_tabu(cov_pool *pool, int32_t slot, int32_t *out);  /* M*n*q       */
int cov_pool_get_rng(cov_pool *pool, int32_t slot, uint64_t *out4);
/* Leader-CTA cycle counts per phase, accumulated over launches (the
 * counterpart of the reference's -DPROF timers, covsearch2e.c:109-131):
 * [0] pick [1] candidates+sample [2] entering side [3] select
 * [4] commit+sphere [5] finish [6] list compaction [7] other ops,
 * [8..23] finer sub-phases, then [24] uncovered-list x candidate-codeword
 * pairs tested. */
int cov_pool_get_prof(cov_pool *pool, int32_t slot, uint64_t *out25);
int cov_pool_get_trace(cov_pool *pool, int32_t slot, cov_move_rec *out,
                       int64_t cap, int64_t *n_out);
/* Clear a COV_ETIMEOUT left by the launch deadline (cov_pool_set_budget): the
 * slot stopped between moves and the next run continues its trajectory
 * exactly.  Other errors are returned unchanged.  No counterpart in the
 * reference, whose processes stop at -t and are restarted from --out. */
int cov_pool_resume(cov_pool *pool, int32_t slot);
int cov_pool_remove(cov_pool *pool, int32_t slot);
int cov_pool_destroy(cov_pool *pool);

/* ------------------------------------------------------------------------
 * Verification and transforms (host buffers in, host buffers out; the
 * *_dev forms take device pointers and a cudaStream_t passed as void*).
 * --------------------------------------------------------------------- */
/* Exact uncovered count of a code at radius R: cov/verify_cov.py:109-152
 * (verify_pure) and :169-230 (verify_numpy) return the same number. */
int cov_verify(int32_t q, int32_t n, int32_t R, const uint8_t *code, int32_t M,
               int64_t *uncovered);
/* Per-word minimum distance to the code (n+1 when M == 0), its histogram
 * hist[0..n+1] and the covering radius: cov/verify_independent.py:144-186
 * (run_mindist).  dist and hist may be NULL. */
int cov_mindist(int32_t q, int32_t n, const uint8_t *code, int32_t M,
                uint8_t *dist, int64_t *hist, int32_t *radius);
/* Coverage multiplicity cnt[x] = #{i : d(x,c_i) <= R} over the code as a
 * multiset, saturated at 65535: the cnt[] of covsearch2e.c:958-967 and the
 * OUT=2 map of cov/gemm2/dct.cu:360-411. */
int cov_count(int32_t q, int32_t n, int32_t R, const uint8_t *code, int32_t M,
              uint16_t *cnt, int64_t *uncovered);
int cov_mindist_dev(int32_t q, int32_t n, const uint8_t *d_code, int32_t M,
                    uint8_t *d_dist, void *stream);
/* d_cnt is updated in aligned 32-bit pairs: it must have room for q^n
 * entries rounded up to an even number. */
int cov_count_dev(int32_t q, int32_t n, int32_t R, const uint8_t *d_code,
                  int32_t M, uint16_t *d_cnt, void *stream);
int64_t cov_count_above_dev(int32_t q, int32_t n, const uint8_t *d_dist,
                            int32_t R, void *stream);
/* ------------------------------------------------------------------------
 * Quotient search: cov/engine/symsearch.c (the process covengine starts as
 * BIN['symsearch'], covengine:654-660) as a pool of instances on the GPU.
 * A code is a union of orbits {(j, e + j) : j in Z_q} of the diagonal
 * translation; the search runs on the q^(n-1) quotient counters with the
 * reference's trajectory.  Arguments are symsearch's -q -n -R -M --orbits
 * -s --kick --stall --cand (symsearch.c:282-310).
 * --------------------------------------------------------------------- */
typedef struct cov_sym cov_sym;

typedef struct {
    int32_t q, n, R, M;
    int32_t orbits;       /* --orbits (0: M / q)                            */
    int32_t kick;         /* --kick   (symsearch default 2)                 */
    uint64_t seed;        /* -s       (12345)                               */
    int64_t stall;        /* --stall  (3000)                                */
    int32_t cand;         /* --cand   (100000)                              */
    int32_t trace;        /* 1 = keep a cov_move_rec per move; its ncw field
                           * holds the candidate sample size                */
    int64_t trace_cap;
} cov_sym_params;

int cov_sym_create(int32_t max_slots, int32_t cluster, cov_sym **out);
int cov_sym_destroy(cov_sym *pool);
int cov_sym_set_budget(cov_sym *pool, double seconds);   /* per-launch wall limit */
/* "grid_eval": 1 spreads the estimates of a pool with one live instance over
 * the whole GPU (one launch per move for them); 0, the default, keeps every
 * move inside the instance's cluster.  Neither changes a trajectory. */
int cov_sym_set_param(cov_sym *pool, const char *name, int64_t value);
/* Orbit count of these parameters, or COV_EINVAL where symsearch exits 2
 * and COV_ERANGE where it exits 3 (symsearch.c:311-333). */
int cov_sym_orbits(const cov_sym_params *prm);
size_t cov_sym_slot_bytes(const cov_sym_params *prm);
/* Add an instance and place its orbits greedily (symsearch.c:340-356). */
int cov_sym_add(cov_sym *pool, const cov_sym_params *prm, int32_t *slot);
int cov_sym_remove(cov_sym *pool, int32_t slot);
/* "cluster" (CTAs per instance, 1..16) or "it_limit" (stop at exactly this
 * iteration count; -1 none).  Neither changes a trajectory. */
int cov_sym_set_slot_param(cov_sym *pool, int32_t slot, const char *name, int64_t value);
/* Advance every instance by up to `moves` iterations (symsearch.c:376-475);
 * an instance stops early once its quotient is covered. */
int cov_sym_run(cov_sym *pool, int64_t moves);
/* it, uncovered and best count QUOTIENT words (SYMRESULT red_uncovered=);
 * the code's uncovered words are q times as many. */
int cov_sym_status(cov_sym *pool, int32_t slot, cov_status *out);
int cov_sym_resume(cov_sym *pool, int32_t slot);          /* after COV_ETIMEOUT */
int cov_sym_get_rep(cov_sym *pool, int32_t slot, uint8_t *out);   /* orbits x (n-1) */
int cov_sym_get_best(cov_sym *pool, int32_t slot, uint8_t *out);  /* orbits x (n-1) */
int cov_sym_get_cnt(cov_sym *pool, int32_t slot, uint16_t *out);  /* q^(n-1)        */
int cov_sym_get_trace(cov_sym *pool, int32_t slot, cov_move_rec *out, int64_t cap,
                      int64_t *n_out);
int cov_sym_get_rng(cov_sym *pool, int32_t slot, uint64_t *out);  /* 4 words        */
/* Diagnostics: leader cycles by phase (0 pick, 1 candidates, 2 sample,
 * 3 estimate op, 4 selection, 5 commit op, 6 orbit ops) and 8 = moves. */
int cov_sym_get_prof(cov_sym *pool, int32_t slot, uint64_t *out);   /* 9 words        */

/* ------------------------------------------------------------------------
 * Transform-engine primitives for one cell (q, n, R): the GPU side of the
 * LNS solver, replacing cov/gemm2/dct.cu's C ABI (dct_init, dct_transform,
 * dct_map_max, dct_map_hist, dct_map_extract, dct_map_read_at,
 * dct_ball_gather, dct_ball_update, dct_count_eq, dct_free;
 * dct.cu:299-504).  Word indices are MSB-first uint32; all buffers are
 * host memory.
 * --------------------------------------------------------------------- */
typedef struct cov_lns cov_lns;
int cov_lns_create(int32_t q, int32_t n, int32_t R, cov_lns **out);
int cov_lns_destroy(cov_lns *h);
/* coverage multiplicity of the m listed words (repeats count) */
int cov_lns_recount(cov_lns *h, const uint32_t *idx, int32_t m);
/* map[x] = #{y : d(x,y) <= R, cnt[y] == target}: target 0 = gain, 1 = loss */
int cov_lns_map(cov_lns *h, int32_t target);
int cov_lns_map_max(cov_lns *h, int32_t *out);
/* counts of map values v >= 1 in bins (v-1)*nbins/vmax, v capped at vmax;
 * 1 <= nbins <= 8192 */
int cov_lns_map_hist(cov_lns *h, int32_t nbins, int32_t vmax, int64_t *hist);
/* positions with map >= thr in increasing index order (at most cap), and
 * how many there are */
int cov_lns_map_extract(cov_lns *h, int32_t thr, int64_t cap, uint32_t *idx, int32_t *val, int64_t *found);
int cov_lns_map_read(cov_lns *h, const uint32_t *idx, int32_t k, int32_t *out);
/* op 0: out[i] = #{y in the ball of idx[i] : cnt[y] == arg};
 * op 1: add arg (+1 or -1) to cnt over the ball of every idx[i], one after
 * another (cov_lns_apply) */
int cov_lns_ball(cov_lns *h, const uint32_t *idx, int32_t k, int32_t op, int32_t arg, int32_t *out);
/* Add sign (+1 or -1) to cnt over the ball of every listed word, one word
 * after another; *uncovered receives #{x : cnt[x] == 0} afterwards. */
int cov_lns_apply(cov_lns *h, const uint32_t *idx, int32_t k, int32_t sign, int64_t *uncovered);
/* Exact peel in the given order (the peel of cov/gemm2/gpuchain.py:325-364,
 * here sequential and exact): a listed codeword is removed (its ball -1)
 * when, at its turn, no word of its ball is covered by it alone; removed[i]
 * = 1 for those.  The uncovered count never changes. */
int cov_lns_peel(cov_lns *h, const uint32_t *idx, int32_t k, uint8_t *removed, int32_t *nremoved,
                 int64_t *uncovered);
/* Lazy greedy placement (the recreate of cov/gemm2/gpuchain.py:193-279):
 * up to `room` words, each one of maximal exact gain (#uncovered words it
 * covers; ties to the lower index), until everything is covered or no word
 * gains.  Bounds come from the gain map: at most cand_cap candidates above a
 * threshold stay on the device, and a persistent cluster kernel re-counts
 * the best bound exactly until it is current, then places it; the host only
 * refreshes the map when the threshold is reached.  placed[] receives the
 * words in order; stats (may be null): refreshes, exact counts. */
int cov_lns_greedy(cov_lns *h, int32_t room, int64_t cand_cap, uint32_t *placed, int32_t *nplaced,
                   int64_t *uncovered, int64_t *stats);
/* The uncovered words (cnt == 0) in increasing index order, at most cap of
 * them, and how many there are (overwrites the map). */
int cov_lns_uncovered(cov_lns *h, int64_t cap, uint32_t *idx, int64_t *found);
/* #{x : cnt[x] == target} */
int cov_lns_count(cov_lns *h, int32_t target, int64_t *out);
int cov_lns_get_cnt(cov_lns *h, uint16_t *out);
int cov_lns_get_map(cov_lns *h, int32_t *out);

/* The finisher of cov/engine/covcount.c (main, :66-216): de-duplicate the
 * m words (first occurrences kept), top up to M distinct words -- with fast,
 * in base-q counting order; else on still-uncovered words chosen as covcount
 * does (64 xorshift64 probes, a linear scan, then any unused word), marking
 * each new word's ball -- and count the uncovered words (-1 with fast).
 * out: M*n digits.  M must not exceed q^n; without fast q^n <= 1.2e9. */
int cov_finish(int32_t q, int32_t n, int32_t R, int32_t M, const uint8_t *code, int32_t m, int32_t fast,
               uint8_t *out, int32_t *words, int64_t *uncovered);
/* cov_mindist_dev without any device allocation, for callers that cannot
 * allocate (their device memory belongs to another allocator, or they run
 * where an allocation is not allowed).  No counterpart in the reference.
 * Its one scratch buffer is a file-scope device array: q^n must be at most
 * 2^26 (else COV_ERANGE); the first call on a device also looks up the
 * array's device address on the host; calls that overlap on the GPU share
 * the array and race. */
int cov_mindist_dev_static(int32_t q, int32_t n, const uint8_t *d_code,
                           int32_t M, uint8_t *d_dist, void *stream);

#ifdef __cplusplus
}
#endif
#endif
