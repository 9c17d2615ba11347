/*
 * oracle.h -- CPU restatement of the reference covering-code search path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library; the
 * product path (coldcase_gb300/) never does.
 *
 * It restates, in plain C, the p5b configuration of the reference engine
 * cov/engine/covsearch2e.c (hoisted offsets, 2-bit min(cnt,2) shadow,
 * shared-sphere evaluation with the uncovered-word list):
 *   - RNG: xoshiro256++ seeded by splitmix64           covsearch2e.c:201-220
 *   - position subsets                                  covsearch2e.c:249-284
 *   - ball marking / rebuild                            covsearch2e.c:353-380, 958-967
 *   - uncovered-word list                               covsearch2e.c:183-193, 287-338
 *   - pick_uncovered (64 probes, then cyclic scan)      covsearch2e.c:973-1016
 *   - candidate collection + Fisher-Yates sample        covsearch2e.c:1339-1402
 *   - shared-sphere evaluation (WALK_POS / UL / NEG)    covsearch2e.c:592-760
 *   - selection with tabu, aspiration, reservoir ties   covsearch2e.c:1503-1522
 *   - commit (sphere walk, mode 1)                      covsearch2e.c:450-493, 562-590
 *   - tabu stamp, improvement, kick                     covsearch2e.c:1525-1579
 *   - initial code: exact-M rebuild, greedy placement,
 *     remove-and-repair descent                         covsearch2e.c:1156-1240
 *   - code-file writer (M distinct words, top-up)       covsearch2e.c:791-853
 * the quotient search (symoracle.c):
 *   - orbit balls, sphere-difference move, estimate,
 *     greedy init, kicks                                symsearch.c:135-475
 * and the verification side:
 *   - verify_pure ball marking                          cov/verify_cov.py:109-152
 *   - run_mindist per-word minimum distance             cov/verify_independent.py:144-186
 *   - run_dilate R-fold axis dilation                   cov/verify_independent.py:128-141
 *   - per-word coverage multiplicity (dct OUT=2)        cov/gemm2/dct.cu:64-99, 360-411
 *
 * Parity of this restatement is pinned against the reference binary built
 * from its own sources (oracle/Makefile `ref`) and against golden vectors
 * produced by the reference's Python verifiers (tests/golden/).
 */
#ifndef COV_ORACLE_H
#define COV_ORACLE_H
#include <stdint.h>
#include "../include/covgpu.h"   /* cov_move_rec, shared trace layout */

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cov_oracle cov_oracle;

/* Search parameters mirror covsearch2e's CLI: -s seed, --tabu, --kick,
 * --stall, --cand, --threads.  Returns NULL on bad parameters. */
cov_oracle *orc_create(int q, int n, int R, int M, uint64_t seed, int tabu,
                       int kick, long long stall, int cand, int threads);
void orc_destroy(cov_oracle *o);

/* Initial code, as covsearch2e main() does it with --in holding m words:
 * m == M -> rebuild; m < M -> greedy placement of the rest (consumes RNG);
 * m > M -> remove-and-repair descent to M.  `random_init` mirrors
 * --random-init.  Returns the uncovered count after initialisation. */
long long orc_init(cov_oracle *o, const uint8_t *code, int m, int random_init);

/* Run up to `max_moves` further moves (stops early at uncovered == 0 or when
 * best <= target, target < 0 = none).  Writes one record per move into
 * `trace` when non-NULL (capacity max_moves).  Returns the number of moves
 * made. */
long long orc_run(cov_oracle *o, long long max_moves, long long target,
                  cov_move_rec *trace);

/* --wide (covsearch2e.c:1353-1376): while the uncovered-word list is
 * valid and short, the candidates are all n(q-1) moves of each codeword at
 * the target distance.  Returns 0, or -1 when out of memory. */
int orc_set_wide(cov_oracle *o, int wide);
/* --fix0 (covsearch2e.c:1241-1253): before orc_init; codeword 0 is moved to
 * 0^n by translating the whole code and never moves again.  -1 if M < 2. */
int orc_set_fix0(cov_oracle *o, int fix0);
/* --sa --t0 --cool --tmin: focused simulated annealing instead of the tabu
 * selection (covsearch2e.c:1408-1441); --noise PERMILLE: that share of the
 * moves is a random sampled move, not evaluated (:1443-1448) */
int orc_set_sa(cov_oracle *o, int sa, double t0, double cool, double tmin);
int orc_set_noise(cov_oracle *o, int permille);
/* --upick (the oldest listed uncovered word) and --ucache (a cache of
 * uncovered words filled by the scan and by commits), covsearch2e.c:978-1012 */
int orc_set_pick(cov_oracle *o, int upick, int ucache);
/* the uncovered-word list: valid flag and length, stale entries included */
void orc_ul_state(const cov_oracle *o, int *valid, int *n);

long long orc_uncovered(const cov_oracle *o);
long long orc_best_uncovered(const cov_oracle *o);
long long orc_iters(const cov_oracle *o);
long long orc_kicks(const cov_oracle *o);
void orc_get_code(const cov_oracle *o, uint8_t *out);       /* M*n */
void orc_get_best(const cov_oracle *o, uint8_t *out);       /* M*n */
void orc_get_cnt(const cov_oracle *o, uint16_t *out);       /* q^n */
void orc_get_tabu(const cov_oracle *o, int32_t *out);       /* M*n*q */
void orc_get_rng(const cov_oracle *o, uint64_t out[4]);
/* the exact delta of every single-coordinate move of codeword i
 * (dvec[p*q+v]; entries with v == c_p are left untouched) */
void orc_eval_codeword(cov_oracle *o, int i, long long *dvec);

/* covsearch2e write_code_n: M distinct words, duplicates dropped, topped up
 * with the lowest unused word indices.  out holds M*n digits. */
int orc_distinct_code(int q, int n, int M, const uint8_t *cw, int nw,
                      uint8_t *out);

/* ---- quotient search (cov/engine/symsearch.c) ----------------------- */
typedef struct sym_oracle sym_oracle;
/* symsearch's -q -n -R -M --orbits -s --kick --stall --cand; NULL where the
 * reference exits 2 or 3 (symsearch.c:311-333).  orbits <= 0: M / q. */
sym_oracle *sym_create(int q, int n, int R, int M, int orbits, uint64_t seed,
                       int kick, long long stall, int cand);
void sym_destroy(sym_oracle *o);
/* greedy orbit placement; returns the uncovered quotient words */
long long sym_init(sym_oracle *o);
/* up to max_moves iterations; trace (capacity max_moves) gets one
 * cov_move_rec per move, with ncw = the candidate sample size */
long long sym_run(sym_oracle *o, long long max_moves, cov_move_rec *trace);
/* OpenMP threads for the estimates (default 1; the trajectory is the same) */
void sym_set_threads(sym_oracle *o, int threads);
long long sym_uncovered(const sym_oracle *o);
long long sym_best_uncovered(const sym_oracle *o);
long long sym_iters(const sym_oracle *o);
long long sym_kicks(const sym_oracle *o);
int sym_orbits(const sym_oracle *o);
void sym_get_rep(const sym_oracle *o, uint8_t *out);    /* orbits x (n-1) */
void sym_get_best(const sym_oracle *o, uint8_t *out);   /* orbits x (n-1) */
void sym_get_cnt(const sym_oracle *o, uint16_t *out);   /* q^(n-1) */
void sym_get_rng(const sym_oracle *o, uint64_t out[4]);

/* ---- verification side ---------------------------------------------- */
/* multiplicity cnt[x] = #{i : d(x, c_i) <= R} (multiset), saturated at 65535 */
int orc_cover_count(int q, int n, int R, const uint8_t *code, int M,
                    uint16_t *cnt);
/* verify_pure: number of words not within R of the (distinct) code */
long long orc_verify_pure(int q, int n, int R, const uint8_t *code, int M);
/* run_mindist: per-word min distance to the code, n+1 if M == 0 */
int orc_mindist(int q, int n, const uint8_t *code, int M, uint8_t *dist,
                int threads);
/* run_dilate: 1 iff every word is within R of the code; covered[] optional */
int orc_linemin(int q, int n, const uint8_t *code, int M, uint8_t *dist, int threads);
int orc_dilate(int q, int n, int R, const uint8_t *code, int M,
               uint8_t *covered);

#ifdef __cplusplus
}
#endif
#endif
