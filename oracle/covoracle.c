/*
 * covoracle.c -- CPU restatement of the reference tabu engine, p5b preset.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  It is the checker for the CUDA
 * engine in coldcase_gb300/csrc and the timed CPU baseline of bench.py; the
 * product never loads it.
 *
 * The algorithm is that of cov/engine/covsearch2e.c run as
 * `--preset p5b` (opt_hoist=1, opt_st=2, opt_eval=2; covsearch2e.c:1090),
 * with or without --wide (orc_set_wide), --fix0 (orc_set_fix0), --sa
 * (orc_set_sa), --noise (orc_set_noise) and --upick / --ucache
 * (orc_set_pick).
 * Each function
 * names the reference lines it restates.  Everything that decides the search
 * trajectory -- RNG consumption order, candidate order, tie-breaking, tabu
 * arithmetic -- is reproduced exactly; what only affects speed (offset
 * hoisting, the 2-bit shadow, the uncovered-word list) is restated as well,
 * so that this file is also a faithful CPU timing baseline.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

/* ---------------------------------------------------------------- RNG --- */
/* xoshiro256++ with splitmix64 seeding: covsearch2e.c:201-220 */
typedef struct { uint64_t s[4]; } orng;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t orng_next(orng *r)
{
    uint64_t *s = r->s;
    uint64_t out = rotl64(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return out;
}

static void orng_seed(orng *r, uint64_t seed)
{
    for (int i = 0; i < 4; i++) {
        seed += 0x9E3779B97F4A7C15ULL;
        uint64_t z = seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        r->s[i] = z ^ (z >> 31);
    }
}

static inline uint64_t orng_mod(orng *r, uint64_t m) { return orng_next(r) % m; }

/* ------------------------------------------------------------- state --- */
#define UL_CAP (1 << 20)            /* covsearch2e.c:188 */

struct cov_oracle {
    int q, n, R, M;
    long long N;
    long long pw[32];               /* pw[j] = q^(n-1-j) */
    uint16_t *cnt;                  /* exact multiplicity */
    uint8_t *st;                    /* 2-bit packed min(cnt,2) */
    long long unc;
    uint8_t *code, *best;
    long long *cidx;
    long long best_unc;
    int nsub;  uint8_t *sub;        /* [n][nsub][rs]: R-subsets avoiding p  */
    int nfsub; uint8_t *fsub;       /* [nfsub][rs]: R-subsets of all n      */
    int rs;                         /* max(R,1): row stride of the tables   */
    long long ppc;                  /* (q-1)^R */
    long long totpat;               /* nsub * ppc */
    long long *ul_idx; uint8_t *ul_dig; uint64_t *ul_bit;
    int ul_n, ul_valid;
    int32_t *tabu;
    orng rng;
    int tenure, kick, cand, threads;
    int wide;                       /* --wide: all n(q-1) moves per codeword */
    int fix0;                       /* --fix0: codeword 0 translated to 0^n and frozen */
    int sa;                         /* --sa: focused simulated annealing (covsearch2e.c:1408-1441) */
    double sa_t0, sa_cool, sa_tmin, sa_T;   /* --t0 --cool --tmin and the temperature */
    int noise;                      /* --noise: per-mille of unevaluated moves (:1443-1448) */
    int upick;                      /* --upick: the oldest listed uncovered word (:978-985) */
    int ucache;                     /* --ucache: a cache of uncovered words (:986-995, :1007-1012) */
    long long ucbuf[4096];          /* the cache (UCCAP, covsearch2e.c:87-90) */
    int ucn;
    size_t cand_cap;                /* entries of ci/cp/cv/cd */
    long long stall;
    long long it, since_improve, nkicks;
    int inited;
    /* per-move scratch */
    int *ci, *cp, *cv, *dist, *cwl, *dv_ep, *of_ep;
    long long *cd, *offs, *dvec;
    long long epoch;
};

static long long ipow_ll(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }

static long long binom_ll(int a, int b)
{
    if (b < 0 || b > a) return 0;
    if (b > a - b) b = a - b;
    long long r = 1;
    for (int i = 0; i < b; i++) r = r * (a - i) / (i + 1);
    return r;
}

/* lexicographic R-subsets of `pool` (size np) into out[k*rs + t];
 * the order of covsearch2e.c:249-284 */
static int fill_subsets(const int *pool, int np, int R, int rs, uint8_t *out)
{
    int c[32];
    int k = 0;
    long long total = binom_ll(np, R);
    if (total <= 0) return 0;
    for (int t = 0; t < R; t++) c[t] = t;
    for (;;) {
        for (int t = 0; t < R; t++) out[(size_t)k * rs + t] = (uint8_t)pool[c[t]];
        k++;
        int t = R - 1;
        while (t >= 0 && c[t] == np - R + t) t--;
        if (t < 0) break;
        c[t]++;
        for (int s = t + 1; s < R; s++) c[s] = c[s - 1] + 1;
    }
    return k;
}

static inline void word_of(const cov_oracle *o, long long x, uint8_t *w)
{
    for (int j = 0; j < o->n; j++) w[j] = (uint8_t)((x / o->pw[j]) % o->q);
}

static inline long long widx(const cov_oracle *o, const uint8_t *w)
{
    long long x = 0;
    for (int j = 0; j < o->n; j++) x += (long long)w[j] * o->pw[j];
    return x;
}

/* offs[j*q + k] = (k-th value != c_j, ascending, minus c_j) * pw[j]:
 * covsearch2e.c:341-347 */
static void make_offs(const cov_oracle *o, const uint8_t *c, long long *offs)
{
    for (int j = 0; j < o->n; j++) {
        int k = 0;
        for (int v = 0; v < o->q; v++)
            if (v != c[j]) offs[(size_t)j * o->q + (k++)] = (long long)(v - c[j]) * o->pw[j];
    }
}

/* 2-bit shadow: covsearch2e.c:95-107 */
static inline int st_get(const cov_oracle *o, long long w)
{
    return (o->st[w >> 2] >> ((w & 3) << 1)) & 3;
}
static inline void st_put(cov_oracle *o, long long w, int c)
{
    if (c > 2) return;
    int sh = (int)((w & 3) << 1);
    uint8_t *b = &o->st[w >> 2];
    *b = (uint8_t)((*b & ~(3 << sh)) | (c << sh));
}

/* ------------------------------------------- uncovered-word list ------- */
/* covsearch2e.c:287-338 */
static inline int ul_has(const cov_oracle *o, long long w) { return (o->ul_bit[w >> 6] >> (w & 63)) & 1; }

static inline void ul_add(cov_oracle *o, long long w)
{
    if (!o->ul_valid || ul_has(o, w)) return;
    if (o->ul_n >= UL_CAP) { o->ul_valid = 0; return; }
    o->ul_bit[w >> 6] |= 1ULL << (w & 63);
    o->ul_idx[o->ul_n] = w;
    word_of(o, w, o->ul_dig + (size_t)o->ul_n * o->n);
    o->ul_n++;
}

static void ul_compact(cov_oracle *o)
{
    int m = 0;
    for (int e = 0; e < o->ul_n; e++) {
        long long w = o->ul_idx[e];
        if (o->cnt[w] == 0) {
            if (m != e) {
                o->ul_idx[m] = w;
                memcpy(o->ul_dig + (size_t)m * o->n, o->ul_dig + (size_t)e * o->n, o->n);
            }
            m++;
        } else {
            o->ul_bit[w >> 6] &= ~(1ULL << (w & 63));
        }
    }
    o->ul_n = m;
}

static void ul_rebuild(cov_oracle *o)
{
    memset(o->ul_bit, 0, (size_t)((o->N + 63) / 64) * 8);
    o->ul_n = 0;
    o->ul_valid = 1;
    for (long long w = 0; w < o->N; w++) {
        if (o->cnt[w]) continue;
        if (o->ul_n >= UL_CAP) { o->ul_valid = 0; return; }
        o->ul_bit[w >> 6] |= 1ULL << (w & 63);
        o->ul_idx[o->ul_n] = w;
        word_of(o, w, o->ul_dig + (size_t)o->ul_n * o->n);
        o->ul_n++;
    }
}

/* ------------------------------------------------- ball marking -------- */
/* +1 / -1 over the whole radius-R ball of c: covsearch2e.c:353-380 */
static long long ball_rec(cov_oracle *o, long long x, const long long *offs,
                          int from, int left, int delta)
{
    long long dunc = 0;
    if (left == 0) return 0;
    for (int j = from; j < o->n; j++) {
        for (int k = 0; k < o->q - 1; k++) {
            long long w = x + offs[(size_t)j * o->q + k];
            if (delta > 0) {
                int c = ++o->cnt[w];
                if (c == 1) dunc--;
                st_put(o, w, c);
            } else {
                int c = --o->cnt[w];
                if (c == 0) { dunc++; ul_add(o, w); }
                st_put(o, w, c);
            }
            dunc += ball_rec(o, w, offs, j + 1, left - 1, delta);
        }
    }
    return dunc;
}

static void ball_apply(cov_oracle *o, const uint8_t *c, long long base, int delta)
{
    long long offs[16 * 16];
    make_offs(o, c, offs);
    long long dunc = 0;
    if (delta > 0) {
        int v = ++o->cnt[base];
        if (v == 1) dunc--;
        st_put(o, base, v);
    } else {
        int v = --o->cnt[base];
        if (v == 0) { dunc++; ul_add(o, base); }
        st_put(o, base, v);
    }
    dunc += ball_rec(o, base, offs, 0, o->R, delta);
    o->unc += dunc;
}

/* words of c's ball that nothing else covers: covsearch2e.c:927-946 */
static long long unique_rec(const cov_oracle *o, long long x, const long long *offs, int from, int left)
{
    long long u = 0;
    if (left == 0) return 0;
    for (int j = from; j < o->n; j++)
        for (int k = 0; k < o->q - 1; k++) {
            long long w = x + offs[(size_t)j * o->q + k];
            u += (o->cnt[w] == 1);
            u += unique_rec(o, w, offs, j + 1, left - 1);
        }
    return u;
}

static long long unique_cover(const cov_oracle *o, const uint8_t *c, long long base)
{
    long long offs[16 * 16];
    make_offs(o, c, offs);
    return (o->cnt[base] == 1) + unique_rec(o, base, offs, 0, o->R);
}

static void st_clear(cov_oracle *o) { memset(o->st, 0, (size_t)((o->N + 3) / 4)); }

/* covsearch2e.c:958-967 */
static void rebuild(cov_oracle *o)
{
    memset(o->cnt, 0, sizeof(uint16_t) * (size_t)o->N);
    st_clear(o);
    o->unc = o->N;
    for (int i = 0; i < o->M; i++) {
        o->cidx[i] = widx(o, o->code + (size_t)i * o->n);
        ball_apply(o, o->code + (size_t)i * o->n, o->cidx[i], +1);
    }
}

/* --------------------------------------------------- sphere walks ------ */
/* One position subset ps[0..R-1] and every assignment of non-centre values
 * to it: the odometer of covsearch2e.c:412-443 / 621-683, last digit fastest.
 * VISIT(w) is evaluated once per word. */
#define SPHERE_SUBSET(o, ps, base, offs, VISIT)                                 \
    do {                                                                        \
        const int R_ = (o)->R, q_ = (o)->q;                                     \
        if (R_ == 0) { long long w = (base); VISIT; break; }                    \
        int k_[16]; long long part_[17];                                        \
        for (int t_ = 0; t_ < R_; t_++) k_[t_] = 0;                             \
        part_[0] = (base);                                                      \
        for (int t_ = 0; t_ < R_ - 1; t_++)                                     \
            part_[t_ + 1] = part_[t_] + (offs)[(size_t)(ps)[t_] * q_];          \
        const long long *last_ = (offs) + (size_t)(ps)[R_ - 1] * q_;            \
        for (;;) {                                                              \
            long long p1_ = part_[R_ - 1];                                      \
            for (int kk_ = 0; kk_ < q_ - 1; kk_++) {                            \
                long long w = p1_ + last_[kk_];                                 \
                VISIT;                                                          \
            }                                                                   \
            int t_ = R_ - 2;                                                    \
            while (t_ >= 0 && k_[t_] == q_ - 2) { k_[t_] = 0; t_--; }           \
            if (t_ < 0) break;                                                  \
            k_[t_]++;                                                           \
            for (int s_ = t_; s_ < R_ - 1; s_++)                                \
                part_[s_ + 1] = part_[s_] + (offs)[(size_t)(ps)[s_] * q_ + k_[s_]]; \
        }                                                                       \
    } while (0)

/* Shared-sphere evaluation of every single-coordinate move of codeword i:
 * covsearch2e.c:592-760.  pos_p = T - H_p from one walk of the full
 * distance-R sphere; neg from the uncovered list (use_ul) or from the
 * per-position walk for the v = u_p entries. */
static void eval_codeword(const cov_oracle *o, int i, const uint8_t *u,
                          const long long *offs, long long *dvec, int use_ul)
{
    const int n = o->n, q = o->q, R = o->R;
    const uint8_t *c = o->code + (size_t)i * n;
    const long long base = o->cidx[i];
    long long T = 0, H[16], neg[16 * 16];
    for (int j = 0; j < n; j++) H[j] = 0;
    memset(neg, 0, sizeof(long long) * (size_t)n * q);

    for (int k = 0; k < o->nfsub; k++) {
        const uint8_t *ps = o->fsub + (size_t)k * o->rs;
        long long t1 = 0;
        SPHERE_SUBSET(o, ps, base, offs, { if (st_get(o, w) == 1) t1++; });
        T += t1;
        for (int t = 0; t < R; t++) H[ps[t]] += t1;
    }

    if (use_ul) {
        int D[17];
        for (int e = 0; e < o->ul_n; e++) {
            long long x = o->ul_idx[e];
            if (o->cnt[x] != 0) continue;
            const uint8_t *xd = o->ul_dig + (size_t)e * n;
            int d = 0;
            for (int j = 0; j < n && d <= R + 1; j++)
                if (xd[j] != c[j]) { if (d < R + 1) D[d] = j; d++; }
            if (d != R + 1) continue;
            for (int t = 0; t <= R; t++) neg[(size_t)D[t] * q + xd[D[t]]]++;
        }
    } else {
        for (int p = 0; p < n; p++) {
            if (c[p] == u[p]) continue;
            long long dv = (long long)(u[p] - c[p]) * o->pw[p];
            long long nn = 0;
            const uint8_t *sp = o->sub + (size_t)p * o->nsub * o->rs;
            for (int k = 0; k < o->nsub; k++) {
                const uint8_t *ps = sp + (size_t)k * o->rs;
                SPHERE_SUBSET(o, ps, base + dv, offs, { nn += (st_get(o, w) == 0); });
            }
            neg[(size_t)p * q + u[p]] = nn;
        }
    }
    for (int p = 0; p < n; p++) {
        long long lv = T - H[p];
        for (int v = 0; v < q; v++)
            if (v != c[p]) dvec[(size_t)p * q + v] = lv - neg[(size_t)p * q + v];
    }
}

/* Commit: covsearch2e.c:450-493 (mode 1) and 562-590.  Leaving word a and
 * entering word a+dv for every pattern of every R-subset avoiding p. */
static long long move_commit(cov_oracle *o, int i, int p, int v)
{
    const int n = o->n;
    uint8_t *c = o->code + (size_t)i * n;
    long long dv = (long long)(v - c[p]) * o->pw[p];
    long long base = o->cidx[i];
    long long offs[16 * 16];
    make_offs(o, c, offs);
    long long dunc = 0;
    const uint8_t *sp = o->sub + (size_t)p * o->nsub * o->rs;
    for (int k = 0; k < o->nsub; k++) {
        const uint8_t *ps = sp + (size_t)k * o->rs;
        SPHERE_SUBSET(o, ps, base, offs, {
            int ca = --o->cnt[w];
            if (ca == 0) {
                dunc++;
                /* --ucache: commits donate newly uncovered words (covsearch2e.c:460, :477) */
                if (o->ucache && o->ucn < 4096) o->ucbuf[o->ucn++] = w;
                ul_add(o, w);
            }
            st_put(o, w, ca);
            int cb = ++o->cnt[w + dv];
            if (cb == 1) dunc--;
            st_put(o, w + dv, cb);
        });
    }
    o->cidx[i] += dv;
    c[p] = (uint8_t)v;
    o->unc += dunc;
    return dunc;
}

/* covsearch2e.c:973-1016 with opt_upick = opt_ucache = 0 */
static long long pick_uncovered(cov_oracle *o)
{
    if (o->upick && o->ul_valid) {
        /* --upick: the list is append-ordered, so its first uncovered entry
         * has been uncovered longest (covsearch2e.c:978-985) */
        for (int e = 0; e < o->ul_n; e++)
            if (o->cnt[o->ul_idx[e]] == 0) return o->ul_idx[e];
    }
    if (o->ucache) {
        /* --ucache: a random cache slot, covered entries discarded (:986-995) */
        while (o->ucn > 0) {
            int j = (int)(orng_next(&o->rng) % (uint64_t)o->ucn);
            long long w = o->ucbuf[j];
            o->ucbuf[j] = o->ucbuf[--o->ucn];
            if (o->cnt[w] == 0) return w;
        }
    }
    for (int t = 0; t < 64; t++) {
        long long w = (long long)(orng_next(&o->rng) % (uint64_t)o->N);
        if (o->cnt[w] == 0) return w;
    }
    long long start = (long long)(orng_next(&o->rng) % (uint64_t)o->N);
    long long found = -1;
    for (long long d = 0; d < o->N; d++) {
        long long w = start + d;
        if (w >= o->N) w -= o->N;
        if (o->cnt[w] == 0) {
            if (!o->ucache) return w;
            /* --ucache: the scan goes on to fill the cache (:1007-1012) */
            if (found < 0) found = w;
            else if (o->ucn < 4096) o->ucbuf[o->ucn++] = w;
            else break;
        }
    }
    return found;
}

/* ------------------------------------------------------ lifecycle ------ */
void orc_destroy(cov_oracle *o)
{
    if (!o) return;
    free(o->cnt); free(o->st); free(o->code); free(o->best); free(o->cidx);
    free(o->sub); free(o->fsub); free(o->ul_idx); free(o->ul_dig); free(o->ul_bit);
    free(o->tabu); free(o->ci); free(o->cp); free(o->cv); free(o->dist);
    free(o->cwl); free(o->dv_ep); free(o->of_ep); free(o->cd); free(o->offs);
    free(o->dvec);
    free(o);
}

cov_oracle *orc_create(int q, int n, int R, int M, uint64_t seed, int tabu,
                       int kick, long long stall, int cand, int threads)
{
    if (q < 2 || q > 16 || n < 1 || n > 16 || R < 0 || M < 1 || M > 65535) return NULL;
    if (R > n) R = n;                 /* balls are the whole space either way */
    cov_oracle *o = calloc(1, sizeof *o);
    if (!o) return NULL;
    o->q = q; o->n = n; o->R = R; o->M = M;
    o->N = ipow_ll(q, n);
    if (o->N > 4000000000LL) { free(o); return NULL; }
    for (int j = 0; j < n; j++) o->pw[j] = ipow_ll(q, n - 1 - j);
    o->tenure = tabu; o->kick = kick; o->stall = stall; o->cand = cand;
    o->threads = threads > 0 ? threads : 1;
    o->rs = R ? R : 1;
    o->ppc = ipow_ll(q - 1, R);
    o->nsub = (int)binom_ll(n - 1, R);
    o->nfsub = (int)binom_ll(n, R);
    o->totpat = (long long)o->nsub * o->ppc;

    o->cnt = calloc((size_t)o->N, sizeof(uint16_t));
    o->st = calloc((size_t)((o->N + 3) / 4), 1);
    o->code = calloc((size_t)M * n, 1);
    o->best = calloc((size_t)M * n, 1);
    o->cidx = calloc((size_t)M, sizeof(long long));
    o->sub = calloc((size_t)n * (o->nsub ? o->nsub : 1) * o->rs, 1);
    o->fsub = calloc((size_t)(o->nfsub ? o->nfsub : 1) * o->rs, 1);
    o->ul_idx = malloc(sizeof(long long) * UL_CAP);
    o->ul_dig = malloc((size_t)UL_CAP * n);
    o->ul_bit = calloc((size_t)((o->N + 63) / 64), 8);
    o->tabu = calloc((size_t)M * n * q, sizeof(int32_t));
    size_t cap = (size_t)M * n;     /* ncand <= (codewords at dtar) * dtar */
    o->cand_cap = cap;
    o->ci = malloc(sizeof(int) * cap); o->cp = malloc(sizeof(int) * cap);
    o->cv = malloc(sizeof(int) * cap); o->cd = malloc(sizeof(long long) * cap);
    o->dist = malloc(sizeof(int) * M); o->cwl = malloc(sizeof(int) * M);
    o->dv_ep = calloc(M, sizeof(int)); o->of_ep = calloc(M, sizeof(int));
    o->offs = malloc(sizeof(long long) * (size_t)M * n * q);
    o->dvec = malloc(sizeof(long long) * (size_t)M * n * q);
    if (!o->cnt || !o->st || !o->code || !o->best || !o->cidx || !o->sub || !o->fsub ||
        !o->ul_idx || !o->ul_dig || !o->ul_bit || !o->tabu || !o->ci || !o->cp || !o->cv ||
        !o->cd || !o->dist || !o->cwl || !o->dv_ep || !o->of_ep || !o->offs || !o->dvec) {
        orc_destroy(o);
        return NULL;
    }
    for (int p = 0; p < n; p++) {
        int pool[32], np = 0;
        for (int j = 0; j < n; j++) if (j != p) pool[np++] = j;
        fill_subsets(pool, np, R, o->rs, o->sub + (size_t)p * o->nsub * o->rs);
    }
    {
        int pool[32];
        for (int j = 0; j < n; j++) pool[j] = j;
        fill_subsets(pool, n, R, o->rs, o->fsub);
    }
    orng_seed(&o->rng, seed);       /* covsearch2e.c:1141 */
    return o;
}

/* covsearch2e.c:1156-1255 (deadline ignored: the oracle always finishes) */
long long orc_init(cov_oracle *o, const uint8_t *code, int m, int random_init)
{
    const int n = o->n, M = o->M;
    int have = 0;
    if (m > M) {
        /* remove-and-repair descent: covsearch2e.c:1163-1192 */
        uint8_t *sc = malloc((size_t)m * n);
        long long *si = malloc(sizeof(long long) * m);
        memcpy(sc, code, (size_t)m * n);
        memset(o->cnt, 0, sizeof(uint16_t) * (size_t)o->N);
        st_clear(o);
        o->unc = o->N;
        for (int i = 0; i < m; i++) {
            si[i] = widx(o, sc + (size_t)i * n);
            ball_apply(o, sc + (size_t)i * n, si[i], +1);
        }
        int ms = m;
        while (ms > M) {
            int worst = 0; long long wu = -1;
            for (int i = 0; i < ms; i++) {
                long long u2 = unique_cover(o, sc + (size_t)i * n, si[i]);
                if (wu < 0 || u2 < wu) { wu = u2; worst = i; }
            }
            ball_apply(o, sc + (size_t)worst * n, si[worst], -1);
            ms--;
            memmove(sc + (size_t)worst * n, sc + (size_t)(worst + 1) * n, (size_t)(ms - worst) * n);
            memmove(si + worst, si + worst + 1, sizeof(long long) * (size_t)(ms - worst));
        }
        memcpy(o->code, sc, (size_t)M * n);
        free(sc); free(si);
        have = M;
    } else if (m > 0) {
        memcpy(o->code, code, (size_t)m * n);
        have = m;
    }
    if (have < M && !random_init) {
        /* greedy placement on uncovered words: covsearch2e.c:1197-1234 */
        memset(o->cnt, 0, sizeof(uint16_t) * (size_t)o->N);
        st_clear(o);
        o->unc = o->N;
        for (int i = 0; i < have; i++) {
            o->cidx[i] = widx(o, o->code + (size_t)i * n);
            ball_apply(o, o->code + (size_t)i * n, o->cidx[i], +1);
        }
        for (int i = have; i < M; i++) {
            long long w = pick_uncovered(o);
            if (w < 0) w = (long long)orng_mod(&o->rng, (uint64_t)o->N);
            word_of(o, w, o->code + (size_t)i * n);
            o->cidx[i] = w;
            ball_apply(o, o->code + (size_t)i * n, o->cidx[i], +1);
        }
    } else {
        for (int i = have; i < M; i++)
            for (int j = 0; j < n; j++)
                o->code[(size_t)i * n + j] = (uint8_t)orng_mod(&o->rng, (uint64_t)o->q);
        rebuild(o);
    }
    if (o->fix0) {
        /* translate the code so that codeword 0 is 0^n (an isometry), then
         * keep it there: covsearch2e.c:1241-1253 */
        uint8_t t0v[16];
        memcpy(t0v, o->code, n);
        for (int i = 0; i < M; i++)
            for (int j = 0; j < n; j++)
                o->code[(size_t)i * n + j] = (uint8_t)((o->code[(size_t)i * n + j] + o->q - t0v[j]) % o->q);
        rebuild(o);
    }
    memcpy(o->best, o->code, (size_t)M * n);
    o->best_unc = o->unc;
    o->ul_valid = 0;                /* built lazily: covsearch2e.c:1139 */
    o->ul_n = 0;
    memset(o->tabu, 0, sizeof(int32_t) * (size_t)M * n * o->q);
    o->it = 0; o->since_improve = 0; o->nkicks = 0;
    o->inited = 1;
    return o->unc;
}

/* The per-iteration loop, covsearch2e.c:1304-1580, for `max_moves` moves. */
long long orc_run(cov_oracle *o, long long max_moves, long long target, cov_move_rec *trace)
{
    if (!o->inited) return -1;
    const int n = o->n, q = o->q, R = o->R, M = o->M;
    uint8_t u[16], tw[16];
    long long done = 0;
    const int par_cand = (o->nsub < 256);          /* covsearch2e.c:1285 */
#ifdef _OPENMP
    omp_set_num_threads(o->threads);
#endif
    while (o->unc > 0 && done < max_moves) {
        if (target >= 0 && o->best_unc <= target) break;
        o->it++;
        done++;
        if (!o->ul_valid && o->unc <= UL_CAP / 2) ul_rebuild(o);
        else if (o->ul_valid && o->ul_n > 2 * o->unc + 64) ul_compact(o);

        long long uw = pick_uncovered(o);
        if (uw < 0) { o->it--; done--; break; }
        word_of(o, uw, u);

        /* candidates: covsearch2e.c:1339-1380 */
        int dmin = n + 1;
        for (int i = o->fix0; i < M; i++) {
            const uint8_t *c = o->code + (size_t)i * n;
            int d = 0;
            for (int j = 0; j < n; j++) d += (c[j] != u[j]);
            o->dist[i] = d;
            if (d < dmin) dmin = d;
        }
        int dtar = (dmin <= R + 1) ? R + 1 : dmin;
        /* --wide: every single-coordinate move of the codewords at dtar,
         * decided before collecting so that candidates and evaluator agree
         * (covsearch2e.c:1353-1376) */
        const int wide_now = o->wide && o->ul_valid &&
                             ((long long)o->ul_n * n < (long long)(R + 1) * o->totpat);
        int ncand = 0;
        for (int i = o->fix0; i < M; i++) {
            if (o->dist[i] != dtar) continue;
            const uint8_t *c = o->code + (size_t)i * n;
            if (wide_now) {
                for (int p = 0; p < n; p++)
                    for (int v = 0; v < q; v++) {
                        if (v == c[p]) continue;
                        o->ci[ncand] = i; o->cp[ncand] = p; o->cv[ncand] = v; ncand++;
                    }
                continue;
            }
            for (int p = 0; p < n; p++) {
                if (c[p] == u[p]) continue;
                o->ci[ncand] = i; o->cp[ncand] = p; o->cv[ncand] = u[p]; ncand++;
            }
        }
        if (ncand == 0) {
            int i = o->fix0 + (int)orng_mod(&o->rng, (uint64_t)(M - o->fix0));
            int p = (int)orng_mod(&o->rng, (uint64_t)n);
            o->ci[0] = i; o->cp[0] = p; o->cv[0] = u[p]; ncand = 1;
        }
        int take = ncand < o->cand ? ncand : o->cand;
        for (int s = 0; s < take; s++) {           /* covsearch2e.c:1383-1389 */
            int j = s + (int)orng_mod(&o->rng, (uint64_t)(ncand - s));
            int ti = o->ci[s], tp = o->cp[s], tv = o->cv[s];
            o->ci[s] = o->ci[j]; o->cp[s] = o->cp[j]; o->cv[s] = o->cv[j];
            o->ci[j] = ti; o->cp[j] = tp; o->cv[j] = tv;
        }
        o->epoch++;
        const int ep = (int)(o->epoch & 0x7fffffff);
        int ncw = 0;
        for (int s = 0; s < take; s++) {
            int i = o->ci[s];
            if (o->of_ep[i] != ep) {
                o->of_ep[i] = ep;
                make_offs(o, o->code + (size_t)i * n, o->offs + (size_t)i * n * q);
            }
            if (o->dv_ep[i] != ep) { o->dv_ep[i] = ep; o->cwl[ncw++] = i; }
        }
        int use_ul = o->ul_valid && ((long long)o->ul_n * n < (long long)(R + 1) * o->totpat);
        if (o->sa) {
            /* focused simulated annealing (covsearch2e.c:1408-1441): one
             * random sampled move, its exact delta, Metropolis acceptance */
            const int s2 = (int)orng_mod(&o->rng, (uint64_t)take);
            const int i = o->ci[s2], p = o->cp[s2], v = o->cv[s2];
            eval_codeword(o, i, u, o->offs + (size_t)i * n * q, o->dvec + (size_t)i * n * q, use_ul);
            const long long d = o->dvec[((size_t)i * n + p) * q + v];
            int accept;
            if (d <= 0) accept = 1;
            else {
                const double pr = exp(-(double)d / o->sa_T);
                accept = (double)(orng_next(&o->rng) >> 11) * 0x1.0p-53 < pr;
            }
            cov_move_rec rec;
            memset(&rec, 0, sizeof rec);
            rec.it = o->it; rec.u = uw; rec.delta = d; rec.ncand = ncand; rec.ncw = 1;
            /* kicked: bit 1 the proposal was rejected, bit 0 the stall reheat */
            rec.i = i; rec.p = p; rec.v = v; rec.kicked = accept ? 0 : 2;
            if (accept) {
                move_commit(o, i, p, v);
                if (o->unc < o->best_unc) {
                    o->best_unc = o->unc;
                    memcpy(o->best, o->code, (size_t)M * n);
                    o->since_improve = 0;
                }
            }
            rec.unc = o->unc;
            o->sa_T *= o->sa_cool;
            if (o->sa_T < o->sa_tmin) o->sa_T = o->sa_t0;      /* reheat */
            if (++o->since_improve > o->stall) {
                o->sa_T = o->sa_t0;
                o->since_improve = 0;
                o->nkicks++;
                rec.kicked |= 1;
            }
            rec.unc_end = o->unc;
            rec.best = o->best_unc;
            if (trace) trace[done - 1] = rec;
            if (o->best_unc == 0) break;
            continue;
        }
        int noisy = 0, ns = 0;
        if (o->noise && (int)orng_mod(&o->rng, 1000) < o->noise) {
            /* covsearch2e.c:1443-1448: a random sampled move, not evaluated */
            noisy = 1;
            ns = (int)orng_mod(&o->rng, (uint64_t)take);
        }
        /* evaluation: covsearch2e.c:1455-1476 */
#pragma omp parallel for schedule(dynamic, 1) if (!noisy && ncw > 1 && par_cand && o->threads > 1)
        for (int z = 0; z < (noisy ? 0 : ncw); z++) {
            int i = o->cwl[z];
            eval_codeword(o, i, u, o->offs + (size_t)i * n * q, o->dvec + (size_t)i * n * q, use_ul);
        }
        for (int s = 0; s < (noisy ? 0 : take); s++)
            o->cd[s] = o->dvec[((size_t)o->ci[s] * n + o->cp[s]) * q + o->cv[s]];

        /* selection: covsearch2e.c:1503-1518 */
        long long bestd = 1LL << 60;
        int nties = 0, bi = -1, bp = -1, bv = -1, bs = -1;
        if (noisy) { bi = o->ci[ns]; bp = o->cp[ns]; bv = o->cv[ns]; bs = ns; }
        for (int s = 0; s < (noisy ? 0 : take); s++) {
            int i = o->ci[s], p = o->cp[s], v = o->cv[s];
            long long d = o->cd[s];
            int is_tabu = o->tabu[((size_t)i * n + p) * q + v] > o->it;
            if (is_tabu && o->unc + d >= o->best_unc) continue;
            if (d < bestd) { bestd = d; bi = i; bp = p; bv = v; bs = s; nties = 1; }
            else if (d == bestd) {
                nties++;
                if (orng_mod(&o->rng, (uint64_t)nties) == 0) { bi = i; bp = p; bv = v; bs = s; }
            }
        }
        if (bi < 0) {
            int s = (int)orng_mod(&o->rng, (uint64_t)take);
            bi = o->ci[s]; bp = o->cp[s]; bv = o->cv[s]; bs = s;
        }
        long long chosen_d = noisy ? 0 : o->cd[bs];
        int oldv = o->code[(size_t)bi * n + bp];
        const long long dunc = move_commit(o, bi, bp, bv);
        if (noisy) chosen_d = dunc;
        o->tabu[((size_t)bi * n + bp) * q + oldv] = (int)(o->it + o->tenure + (long long)orng_mod(&o->rng, 4));

        cov_move_rec rec;
        memset(&rec, 0, sizeof rec);
        rec.it = o->it; rec.u = uw; rec.delta = chosen_d; rec.unc = o->unc;
        rec.ncand = ncand; rec.ncw = ncw; rec.i = bi; rec.p = bp; rec.v = bv;

        if (o->unc < o->best_unc) {
            o->best_unc = o->unc;
            memcpy(o->best, o->code, (size_t)M * n);
            o->since_improve = 0;
        } else if (++o->since_improve > o->stall) {
            /* kick: covsearch2e.c:1553-1579 */
            for (int t = 0; t < o->kick; t++) {
                int i = o->fix0 + (int)orng_mod(&o->rng, (uint64_t)(M - o->fix0));
                uint8_t *c = o->code + (size_t)i * n;
                ball_apply(o, c, o->cidx[i], -1);
                long long w = pick_uncovered(o);
                if (w >= 0) {
                    word_of(o, w, tw);
                    memcpy(c, tw, n);
                    for (int t2 = 0; t2 < R; t2++) {
                        /* gcc sequences the assigned value's draw before the
                         * subscript's draw in covsearch2e.c:1567 */
                        uint8_t val = (uint8_t)orng_mod(&o->rng, (uint64_t)q);
                        int pos = (int)orng_mod(&o->rng, (uint64_t)n);
                        c[pos] = val;
                    }
                } else {
                    for (int j = 0; j < n; j++) c[j] = (uint8_t)orng_mod(&o->rng, (uint64_t)q);
                }
                o->cidx[i] = widx(o, c);
                ball_apply(o, c, o->cidx[i], +1);
            }
            o->nkicks++;
            memset(o->tabu, 0, sizeof(int32_t) * (size_t)M * n * q);
            o->since_improve = 0;
            rec.kicked = 1;
        }
        rec.unc_end = o->unc;
        rec.best = o->best_unc;
        if (trace) trace[done - 1] = rec;
        if (o->best_unc == 0) break;
    }
    return done;
}

/* --wide (covsearch2e.c:1076): the candidate arrays grow to M*n*(q-1) */
int orc_set_wide(cov_oracle *o, int wide)
{
    const size_t cap = wide ? (size_t)o->M * o->n * (o->q - 1) : (size_t)o->M * o->n;
    if (cap > o->cand_cap) {
        int *ci = realloc(o->ci, sizeof(int) * cap);
        if (ci) o->ci = ci;
        int *cp = realloc(o->cp, sizeof(int) * cap);
        if (cp) o->cp = cp;
        int *cv = realloc(o->cv, sizeof(int) * cap);
        if (cv) o->cv = cv;
        long long *cd = realloc(o->cd, sizeof(long long) * cap);
        if (cd) o->cd = cd;
        if (!ci || !cp || !cv || !cd) return -1;
        o->cand_cap = cap;
    }
    o->wide = wide ? 1 : 0;
    return 0;
}

/* --sa --t0 --cool --tmin (covsearch2e.c:1034-1035, :1061-1064) */
int orc_set_sa(cov_oracle *o, int sa, double t0, double cool, double tmin)
{
    o->sa = sa ? 1 : 0;
    o->sa_t0 = t0; o->sa_cool = cool; o->sa_tmin = tmin; o->sa_T = t0;
    return 0;
}

/* --noise PERMILLE (covsearch2e.c:1032, :1056) */
int orc_set_noise(cov_oracle *o, int permille)
{
    o->noise = permille;        /* any value: a nonzero one draws the coin */
    return 0;
}

/* --upick / --ucache (covsearch2e.c:1075-1076, :1145); set before orc_init */
int orc_set_pick(cov_oracle *o, int upick, int ucache)
{
    o->upick = upick ? 1 : 0;
    o->ucache = ucache ? 1 : 0;
    o->ucn = 0;
    return 0;
}

/* --fix0 (covsearch2e.c:1074, :1241-1253); set before orc_init */
int orc_set_fix0(cov_oracle *o, int fix0)
{
    if (fix0 && o->M < 2) return -1;
    o->fix0 = fix0 ? 1 : 0;
    return 0;
}

void orc_ul_state(const cov_oracle *o, int *valid, int *n)
{
    *valid = o->ul_valid;
    *n = o->ul_n;
}

long long orc_uncovered(const cov_oracle *o) { return o->unc; }
long long orc_best_uncovered(const cov_oracle *o) { return o->best_unc; }
long long orc_iters(const cov_oracle *o) { return o->it; }
long long orc_kicks(const cov_oracle *o) { return o->nkicks; }
void orc_get_code(const cov_oracle *o, uint8_t *out) { memcpy(out, o->code, (size_t)o->M * o->n); }
void orc_get_best(const cov_oracle *o, uint8_t *out) { memcpy(out, o->best, (size_t)o->M * o->n); }
void orc_get_cnt(const cov_oracle *o, uint16_t *out) { memcpy(out, o->cnt, sizeof(uint16_t) * (size_t)o->N); }
void orc_get_tabu(const cov_oracle *o, int32_t *out)
{
    memcpy(out, o->tabu, sizeof(int32_t) * (size_t)o->M * o->n * o->q);
}
void orc_get_rng(const cov_oracle *o, uint64_t out[4]) { memcpy(out, o->rng.s, 32); }

void orc_eval_codeword(cov_oracle *o, int i, long long *dvec)
{
    /* the full dvec needs the uncovered list (every (p,v) entry) */
    if (!o->ul_valid) ul_rebuild(o);
    long long offs[16 * 16];
    uint8_t u[16];
    memcpy(u, o->code + (size_t)i * o->n, o->n);
    make_offs(o, o->code + (size_t)i * o->n, offs);
    if (o->ul_valid) {
        eval_codeword(o, i, u, offs, dvec, 1);
    }
}

/* covsearch2e.c:791-837: M distinct words, duplicates dropped in order,
 * topped up with the lowest unused indices. */
int orc_distinct_code(int q, int n, int M, const uint8_t *cw, int nw, uint8_t *out)
{
    long long N = ipow_ll(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipow_ll(q, n - 1 - j);
    if (nw > M) nw = M;
    long long *ix = malloc(sizeof(long long) * (size_t)(M > 0 ? M : 1));
    if (!ix) return -1;
    int m = 0;
    for (int i = 0; i < nw; i++) {
        long long x = 0;
        for (int j = 0; j < n; j++) x += (long long)cw[(size_t)i * n + j] * pw[j];
        int dup = 0;
        for (int k = 0; k < m; k++) if (ix[k] == x) { dup = 1; break; }
        if (dup) continue;
        memcpy(out + (size_t)m * n, cw + (size_t)i * n, n);
        ix[m++] = x;
    }
    for (long long x = 0; m < M && x < N; x++) {
        int dup = 0;
        for (int k = 0; k < m; k++) if (ix[k] == x) { dup = 1; break; }
        if (dup) continue;
        for (int j = 0; j < n; j++) out[(size_t)m * n + j] = (uint8_t)((x / pw[j]) % q);
        ix[m++] = x;
    }
    free(ix);
    return m;
}
