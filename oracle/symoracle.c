/*
 * symoracle.c -- CPU restatement of the reference quotient search.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  It is the checker for the CUDA
 * quotient engine in coldcase_gb300/csrc/cov_sym.cu and the CPU baseline of
 * bench.py's quotient leg; the product never loads it.
 *
 * The algorithm is cov/engine/symsearch.c: local search over codes that are
 * unions of orbits of the diagonal translation x -> x + 1^n, carried out in
 * the quotient Z_q^(n-1).  An orbit with representative e (first coordinate
 * 0) covers the quotient word d with multiplicity
 *     #{delta : #{i : d_i != e_i + delta} <= R - [delta != 0]}
 * (symsearch.c:15-31), i.e. it is one ball of radius R around e plus q-1
 * balls of radius R-1 around e + delta*1.  Everything that decides the
 * trajectory -- RNG consumption, candidate order, the read-only estimate of
 * a move, tie-breaking, kicks -- follows the reference; each function names
 * the lines it restates.  The reference stops on a wall-clock limit only;
 * here the caller gives a move budget, so a reference run of K iterations is
 * replayed as K moves.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

typedef struct { uint64_t s[4]; } srng;

static inline uint64_t s_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* xoshiro256++ and splitmix64 seeding, symsearch.c:77-84 */
static inline uint64_t s_next(srng *r)
{
    uint64_t *s = r->s;
    uint64_t out = s_rotl(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = s_rotl(s[3], 45);
    return out;
}

static void s_seed(srng *r, uint64_t seed)
{
    for (int i = 0; i < 4; i++) {
        seed += 0x9E3779B97F4A7C15ULL;
        uint64_t z = seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        r->s[i] = z ^ (z >> 31);
    }
}

static inline uint64_t s_mod(srng *r, uint64_t m) { return s_next(r) % m; }

struct sym_oracle {
    int q, n, R, NR, norb, kick, cand;
    int threads;                     /* OpenMP threads for the estimates */
    long long stall;
    long long N;                     /* q^(n-1) quotient words */
    long long pw[32];
    uint16_t *cnt;
    uint8_t *rep, *best;             /* norb x NR representatives (first coordinate 0 dropped) */
    long long *cidx;                 /* norb x q: index of centre e + delta */
    long long unc, best_unc;
    long long it, since_improve, nkicks;
    int inited;
    /* R-subsets (and (R-1)-subsets) of the NR-1 positions other than p:
     * sub[r][p][k][.] (symsearch.c:91-112) */
    int ncomb[2];
    uint8_t *sub[2];
    srng rng;
    /* per-move scratch */
    int *ci, *cp, *cv;
    long long *cd;
    uint8_t *cen;
};

static long long s_ipow(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }

static long long s_binom(int a, int b)
{
    if (b < 0 || b > a) return 0;
    long long r = 1;
    if (b > a - b) b = a - b;
    for (int i = 0; i < b; i++) r = r * (a - i) / (i + 1);
    return r;
}

/* lexicographic r-subsets of the positions other than p, per p */
static uint8_t *s_subsets(int NR, int r, int *count)
{
    const int nc = (int)s_binom(NR - 1, r), rs = r ? r : 1;
    uint8_t *out = calloc((size_t)NR * (nc ? nc : 1) * rs, 1);
    if (!out) return NULL;
    for (int p = 0; p < NR; p++) {
        int pool[32], np = 0, c[16];
        for (int j = 0; j < NR; j++) if (j != p) pool[np++] = j;
        for (int i = 0; i < r; i++) c[i] = i;
        for (int k = 0; k < nc; k++) {
            for (int i = 0; i < r; i++) out[((size_t)p * nc + k) * rs + i] = (uint8_t)pool[c[i]];
            int i = r - 1;
            while (i >= 0 && c[i] == np - r + i) i--;
            if (i < 0) break;
            c[i]++;
            for (int j = i + 1; j < r; j++) c[j] = c[j - 1] + 1;
        }
    }
    *count = nc;
    return out;
}

static long long s_widx(const sym_oracle *o, const uint8_t *w)
{
    long long x = 0;
    for (int j = 0; j < o->NR; j++) x += (long long)w[j] * o->pw[j];
    return x;
}

static void s_word(const sym_oracle *o, long long x, uint8_t *w)
{
    for (int j = 0; j < o->NR; j++) w[j] = (uint8_t)((x / o->pw[j]) % o->q);
}

/* the whole radius-rad ball of c, +1 or -1 (symsearch.c:135-159) */
static long long s_ball_rec(sym_oracle *o, long long x, const uint8_t *c, int from, int left, int delta)
{
    long long du = 0;
    if (left == 0) return 0;
    for (int j = from; j < o->NR; j++)
        for (int v = 0; v < o->q; v++) {
            if (v == c[j]) continue;
            long long w = x + (long long)(v - c[j]) * o->pw[j];
            if (delta > 0) { if (o->cnt[w]++ == 0) du--; }
            else if (--o->cnt[w] == 0) du++;
            du += s_ball_rec(o, w, c, j + 1, left - 1, delta);
        }
    return du;
}

static void s_ball(sym_oracle *o, const uint8_t *c, long long base, int rad, int delta)
{
    if (rad < 0) return;
    long long du = 0;
    if (delta > 0) { if (o->cnt[base]++ == 0) du--; }
    else if (--o->cnt[base] == 0) du++;
    du += s_ball_rec(o, base, c, 0, rad, delta);
    o->unc += du;
}

/* all q balls of orbit i (symsearch.c:162-174) */
static void s_orbit(sym_oracle *o, int i, int delta)
{
    uint8_t c[32];
    for (int d = 0; d < o->q; d++) {
        const int rad = o->R - (d != 0);
        if (rad < 0) continue;
        for (int j = 0; j < o->NR; j++) c[j] = (uint8_t)((o->rep[(size_t)i * o->NR + j] + d) % o->q);
        const long long b = s_widx(o, c);
        o->cidx[(size_t)i * o->q + d] = b;
        s_ball(o, c, b, rad, delta);
    }
}

/* One R'-subset of the positions other than p: every word a that differs
 * from centre c exactly there (values other than c's), paired with
 * b = a + dv (position p moved).  mode 0 counts (cnt[a]==1) - (cnt[b]==0);
 * mode 1 applies the move (symsearch.c:177-205). */
static long long s_walk(sym_oracle *o, const uint8_t *ps, const uint8_t *c, long long base, long long dv,
                        int rad, int mode, int at)
{
    if (at == rad) {
        const long long a = base, b = base + dv;
        long long du = 0;
        if (mode) {
            if (--o->cnt[a] == 0) du++;
            if (o->cnt[b]++ == 0) du--;
        } else {
            if (o->cnt[a] == 1) du++;
            if (o->cnt[b] == 0) du--;
        }
        return du;
    }
    long long du = 0;
    const int j = ps[at];
    for (int v = 0; v < o->q; v++) {
        if (v == c[j]) continue;
        du += s_walk(o, ps, c, base + (long long)(v - c[j]) * o->pw[j], dv, rad, mode, at + 1);
    }
    return du;
}

/* Move orbit i: rep[i][p] -> v, i.e. every centre e + delta moves its p-th
 * digit to v + delta.  mode 0 is the reference's read-only estimate (each
 * sub-move judged against the unchanged counters), mode 1 the exact commit
 * (symsearch.c:207-245). */
static long long s_move(sym_oracle *o, int i, int p, int v, int mode)
{
    long long du = 0;
    uint8_t c[32];
    for (int d = 0; d < o->q; d++) {
        const int rad = o->R - (d != 0);
        if (rad < 0) continue;
        for (int j = 0; j < o->NR; j++) c[j] = (uint8_t)((o->rep[(size_t)i * o->NR + j] + d) % o->q);
        const long long base = o->cidx[(size_t)i * o->q + d];
        const int nv = (v + d) % o->q;
        const long long dv = (long long)(nv - c[p]) * o->pw[p];
        const int t = rad == o->R ? 0 : 1, rs = rad ? rad : 1;
        const uint8_t *cb = o->sub[t] + (size_t)p * o->ncomb[t] * rs;
        for (int k = 0; k < o->ncomb[t]; k++) du += s_walk(o, cb + (size_t)k * rs, c, base, dv, rad, mode, 0);
        if (mode) o->cidx[(size_t)i * o->q + d] = base + dv;
    }
    if (mode) {
        o->rep[(size_t)i * o->NR + p] = (uint8_t)v;
        o->unc += du;
    }
    return du;
}

/* 64 uniform probes, then the first zero cyclically after a random start
 * (symsearch.c:268-280) */
static long long s_pick(sym_oracle *o)
{
    for (int t = 0; t < 64; t++) {
        const long long w = (long long)s_mod(&o->rng, (uint64_t)o->N);
        if (o->cnt[w] == 0) return w;
    }
    const long long start = (long long)s_mod(&o->rng, (uint64_t)o->N);
    for (long long d = 0; d < o->N; d++) {
        long long w = start + d;
        if (w >= o->N) w -= o->N;
        if (o->cnt[w] == 0) return w;
    }
    return -1;
}

void sym_destroy(sym_oracle *o)
{
    if (!o) return;
    free(o->cnt); free(o->rep); free(o->best); free(o->cidx);
    free(o->sub[0]); free(o->sub[1]);
    free(o->ci); free(o->cp); free(o->cv); free(o->cd); free(o->cen);
    free(o);
}

/* Arguments and limits of symsearch.c:311-333; orbits <= 0 means M / q. */
sym_oracle *sym_create(int q, int n, int R, int M, int orbits, uint64_t seed, int kick, long long stall,
                       int cand)
{
    if (q < 2 || q > 16 || n < 2 || n > 16 || R < 0 || R > 7 || M < q) return NULL;
    const int norb = orbits > 0 ? orbits : M / q;
    if (norb < 1 || norb > M / q) return NULL;
    if ((long long)norb * q > 65000) return NULL;
    sym_oracle *o = calloc(1, sizeof *o);
    if (!o) return NULL;
    o->q = q; o->n = n; o->R = R; o->NR = n - 1; o->norb = norb;
    o->kick = kick; o->stall = stall; o->cand = cand;
    o->threads = 1;
    o->N = s_ipow(q, o->NR);
    if (o->N > 4000000000LL) { free(o); return NULL; }
    for (int p = 0; p < o->NR; p++) o->pw[p] = s_ipow(q, o->NR - 1 - p);
    o->cnt = calloc((size_t)o->N, sizeof(uint16_t));
    o->rep = calloc((size_t)norb * o->NR, 1);
    o->best = calloc((size_t)norb * o->NR, 1);
    o->cidx = calloc((size_t)norb * q, sizeof(long long));
    o->sub[0] = s_subsets(o->NR, R, &o->ncomb[0]);
    o->sub[1] = R >= 1 ? s_subsets(o->NR, R - 1, &o->ncomb[1]) : calloc(1, 1);
    const size_t maxc = (size_t)norb * q * o->NR + 8;
    o->ci = malloc(sizeof(int) * maxc); o->cp = malloc(sizeof(int) * maxc);
    o->cv = malloc(sizeof(int) * maxc); o->cd = malloc(sizeof(long long) * maxc);
    o->cen = malloc((size_t)norb * q * o->NR);
    if (!o->cnt || !o->rep || !o->best || !o->cidx || !o->sub[0] || !o->sub[1] || !o->ci || !o->cp ||
        !o->cv || !o->cd || !o->cen) {
        sym_destroy(o);
        return NULL;
    }
    s_seed(&o->rng, seed * 0x9E3779B97F4A7C15ULL + 12345);       /* symsearch.c:338 */
    return o;
}

/* Greedy placement: each representative on a still-uncovered quotient word
 * (symsearch.c:340-356; the wall-clock cut of the reference is not
 * restated -- a run long enough for it to act is not replayable). */
long long sym_init(sym_oracle *o)
{
    uint8_t w8[32];
    memset(o->cnt, 0, sizeof(uint16_t) * (size_t)o->N);
    o->unc = o->N;
    for (int i = 0; i < o->norb; i++) {
        long long w = s_pick(o);
        if (w < 0) w = (long long)s_mod(&o->rng, (uint64_t)o->N);
        s_word(o, w, w8);
        memcpy(o->rep + (size_t)i * o->NR, w8, o->NR);
        s_orbit(o, i, +1);
    }
    memcpy(o->best, o->rep, (size_t)o->norb * o->NR);
    o->best_unc = o->unc;
    o->it = o->since_improve = o->nkicks = 0;
    o->inited = 1;
    return o->unc;
}

/* Up to max_moves iterations of symsearch.c:376-475; stops early when the
 * quotient is covered.  One record per move when trace != NULL (ncw holds
 * the sample size). */
long long sym_run(sym_oracle *o, long long max_moves, cov_move_rec *trace)
{
    if (!o->inited) return -1;
    const int q = o->q, NR = o->NR, R = o->R, norb = o->norb;
    uint8_t u[32], tw[32];
    long long done = 0;
    while (o->unc > 0 && done < max_moves) {
        o->it++;
        done++;
        const long long uw = s_pick(o);
        if (uw < 0) { o->it--; done--; break; }
        s_word(o, uw, u);
        /* effective distance of every (orbit, delta) centre (:388-404) */
        int dmin = o->n + 2;
        for (int i = 0; i < norb; i++)
            for (int d = 0; d < q; d++) {
                if (R - (d != 0) < 0) continue;
                uint8_t *cb = o->cen + ((size_t)i * q + d) * NR;
                int dd = 0;
                for (int j = 0; j < NR; j++) {
                    cb[j] = (uint8_t)((o->rep[(size_t)i * NR + j] + d) % q);
                    dd += cb[j] != u[j];
                }
                const int eff = dd + (d != 0);
                if (eff < dmin) dmin = eff;
            }
        const int dtar = dmin <= R + 1 ? R + 1 : dmin;
        /* candidates: orbit, position, the value that puts that centre's
         * digit on u's (:406-418) */
        int nc = 0;
        for (int i = 0; i < norb; i++)
            for (int d = 0; d < q; d++) {
                if (R - (d != 0) < 0) continue;
                const uint8_t *cb = o->cen + ((size_t)i * q + d) * NR;
                int dd = 0;
                for (int j = 0; j < NR; j++) dd += cb[j] != u[j];
                if (dd + (d != 0) != dtar) continue;
                for (int p = 0; p < NR; p++) {
                    if (cb[p] == u[p]) continue;
                    o->ci[nc] = i; o->cp[nc] = p; o->cv[nc] = (u[p] - d + q) % q; nc++;
                }
            }
        if (nc == 0) {                                 /* :419-424 */
            o->ci[0] = (int)s_mod(&o->rng, (uint64_t)norb);
            o->cp[0] = (int)s_mod(&o->rng, (uint64_t)NR);
            o->cv[0] = (int)s_mod(&o->rng, (uint64_t)q);
            nc = 1;
        }
        const int take = nc < o->cand ? nc : o->cand;
        for (int s = 0; s < take; s++) {               /* :425-430 */
            const int j = s + (int)s_mod(&o->rng, (uint64_t)(nc - s));
            int a = o->ci[s], b = o->cp[s], c = o->cv[s];
            o->ci[s] = o->ci[j]; o->cp[s] = o->cp[j]; o->cv[s] = o->cv[j];
            o->ci[j] = a; o->cp[j] = b; o->cv[j] = c;
        }
        /* the estimates only read the counters, so they run in parallel
         * (symsearch.c:432-433); the trajectory does not depend on it */
#pragma omp parallel for schedule(dynamic, 1) if (take > 3 && o->threads > 1) num_threads(o->threads)
        for (int s = 0; s < take; s++) o->cd[s] = s_move(o, o->ci[s], o->cp[s], o->cv[s], 0);
        /* reservoir selection (:436-445) */
        int bi = -1, bp = -1, bv = -1, nties = 0, bs = -1;
        long long bestd = 1LL << 60;
        for (int s = 0; s < take; s++) {
            if (o->cv[s] == o->rep[(size_t)o->ci[s] * NR + o->cp[s]]) continue;
            if (o->cd[s] < bestd) {
                bestd = o->cd[s]; bi = o->ci[s]; bp = o->cp[s]; bv = o->cv[s]; bs = s; nties = 1;
            } else if (o->cd[s] == bestd) {
                nties++;
                if (s_mod(&o->rng, (uint64_t)nties) == 0) { bi = o->ci[s]; bp = o->cp[s]; bv = o->cv[s]; bs = s; }
            }
        }
        if (bi < 0) {
            const int s = (int)s_mod(&o->rng, (uint64_t)take);
            bi = o->ci[s]; bp = o->cp[s]; bv = o->cv[s]; bs = s;
            if (bv == o->rep[(size_t)bi * NR + bp]) bv = (bv + 1) % q;
        }
        const long long est = o->cd[bs];
        s_move(o, bi, bp, bv, 1);
        cov_move_rec rec;
        memset(&rec, 0, sizeof rec);
        rec.it = o->it; rec.u = uw; rec.delta = est; rec.unc = o->unc;
        rec.ncand = nc; rec.ncw = take; rec.i = bi; rec.p = bp; rec.v = bv;
        if (o->unc < o->best_unc) {                   /* :449-458 */
            o->best_unc = o->unc;
            memcpy(o->best, o->rep, (size_t)norb * NR);
            o->since_improve = 0;
        } else if (++o->since_improve > o->stall) {    /* :459-475 */
            for (int t = 0; t < o->kick; t++) {
                const int i = (int)s_mod(&o->rng, (uint64_t)norb);
                s_orbit(o, i, -1);
                const long long w = s_pick(o);
                uint8_t *e = o->rep + (size_t)i * NR;
                if (w >= 0) {
                    s_word(o, w, tw);
                    memcpy(e, tw, NR);
                    for (int t2 = 0; t2 < R; t2++) {
                        /* the assigned value is drawn before the subscript,
                         * as gcc sequences symsearch.c:467 */
                        const uint8_t val = (uint8_t)s_mod(&o->rng, (uint64_t)q);
                        const int pos = (int)s_mod(&o->rng, (uint64_t)NR);
                        e[pos] = val;
                    }
                } else {
                    for (int j = 0; j < NR; j++) e[j] = (uint8_t)s_mod(&o->rng, (uint64_t)q);
                }
                s_orbit(o, i, +1);
            }
            o->nkicks++;
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

void sym_set_threads(sym_oracle *o, int threads) { o->threads = threads > 0 ? threads : 1; }
long long sym_uncovered(const sym_oracle *o) { return o->unc; }
long long sym_best_uncovered(const sym_oracle *o) { return o->best_unc; }
long long sym_iters(const sym_oracle *o) { return o->it; }
long long sym_kicks(const sym_oracle *o) { return o->nkicks; }
int sym_orbits(const sym_oracle *o) { return o->norb; }
void sym_get_rep(const sym_oracle *o, uint8_t *out) { memcpy(out, o->rep, (size_t)o->norb * o->NR); }
void sym_get_best(const sym_oracle *o, uint8_t *out) { memcpy(out, o->best, (size_t)o->norb * o->NR); }
void sym_get_cnt(const sym_oracle *o, uint16_t *out) { memcpy(out, o->cnt, sizeof(uint16_t) * (size_t)o->N); }
void sym_get_rng(const sym_oracle *o, uint64_t out[4]) { memcpy(out, o->rng.s, 32); }
