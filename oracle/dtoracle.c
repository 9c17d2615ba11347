/*
 * dtoracle.c -- CPU restatement of the reference's verification side.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): checker for the coverage-count and
 * distance-transform kernels, and the CPU baseline of bench.py.
 *
 *   orc_cover_count   multiplicity of coverage per word, as covsearch2e's
 *                     rebuild() leaves it in cnt[] (covsearch2e.c:353-380,
 *                     958-967) and as dct.cu's OUT=2 transform writes it
 *                     (cov/gemm2/dct.cu:64-99, 360-411)
 *   orc_verify_pure   cov/verify_cov.py:109-152 (distinct code, ball marking)
 *   orc_mindist       cov/verify_independent.py:144-186 (per-word minimum
 *                     distance, initialised to n+1)
 *   orc_dilate        cov/verify_independent.py:128-141 (R rounds of n
 *                     axis-OR dilations of the code's indicator)
 *   orc_linemin       the same per-word minimum distance as orc_mindist by
 *                     n axis passes of the line-min recurrence
 *                     D(x) = min(D(x), 1 + min over the line of axis j
 *                     through x) on uint8 values -- the CPU form of the
 *                     GPU transform, timed as its CPU baseline (OpenMP over
 *                     the lines of an axis)
 */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "oracle.h"

static long long ipw(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }

/* every word within distance `left` of x by changing positions >= from */
static void mark_rec(uint16_t *cnt, uint8_t *flag, long long x, const uint8_t *c,
                     const long long *pw, int q, int n, int from, int left)
{
    if (left == 0) return;
    for (int j = from; j < n; j++) {
        long long b = x - (long long)c[j] * pw[j];
        for (int v = 0; v < q; v++) {
            if (v == c[j]) continue;
            long long w = b + (long long)v * pw[j];
            if (cnt && cnt[w] != 65535) cnt[w]++;
            if (flag) flag[w] = 1;
            mark_rec(cnt, flag, w, c, pw, q, n, j + 1, left - 1);
        }
    }
}

int orc_cover_count(int q, int n, int R, const uint8_t *code, int M, uint16_t *cnt)
{
    if (q < 2 || n < 1 || R < 0) return -1;
    long long N = ipw(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipw(q, n - 1 - j);
    if (R > n) R = n;
    memset(cnt, 0, sizeof(uint16_t) * (size_t)N);
    for (int i = 0; i < M; i++) {
        const uint8_t *c = code + (size_t)i * n;
        long long x = 0;
        for (int j = 0; j < n; j++) x += (long long)c[j] * pw[j];
        if (cnt[x] != 65535) cnt[x]++;
        mark_rec(cnt, NULL, x, c, pw, q, n, 0, R);
    }
    return 0;
}

long long orc_verify_pure(int q, int n, int R, const uint8_t *code, int M)
{
    long long N = ipw(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipw(q, n - 1 - j);
    if (R > n) R = n;
    uint8_t *cov = calloc((size_t)N, 1);
    if (!cov) return -1;
    for (int i = 0; i < M; i++) {
        const uint8_t *c = code + (size_t)i * n;
        long long x = 0;
        for (int j = 0; j < n; j++) x += (long long)c[j] * pw[j];
        cov[x] = 1;
        mark_rec(NULL, cov, x, c, pw, q, n, 0, R);
    }
    long long unc = 0;
    for (long long x = 0; x < N; x++) unc += !cov[x];
    free(cov);
    return unc;
}

int orc_mindist(int q, int n, const uint8_t *code, int M, uint8_t *dist, int threads)
{
    long long N = ipw(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipw(q, n - 1 - j);
    (void)threads;
#pragma omp parallel for schedule(static) if (threads > 1) num_threads(threads > 0 ? threads : 1)
    for (long long x = 0; x < N; x++) {
        uint8_t w[16];
        for (int j = 0; j < n; j++) w[j] = (uint8_t)((x / pw[j]) % q);
        int best = n + 1;
        for (int i = 0; i < M && best > 0; i++) {
            const uint8_t *c = code + (size_t)i * n;
            int d = 0;
            for (int j = 0; j < n; j++) d += (c[j] != w[j]);
            if (d < best) best = d;
        }
        dist[x] = (uint8_t)best;
    }
    return 0;
}

int orc_linemin(int q, int n, const uint8_t *code, int M, uint8_t *dist, int threads)
{
    long long N = ipw(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipw(q, n - 1 - j);
    const uint8_t inf = (uint8_t)(n + 1);
    memset(dist, inf, (size_t)N);
    for (int i = 0; i < M; i++) {
        long long x = 0;
        for (int j = 0; j < n; j++) x += (long long)code[(size_t)i * n + j] * pw[j];
        dist[x] = 0;
    }
    if (threads < 1) threads = 1;
    for (int j = 0; j < n; j++) {
        /* lines of axis j: (q^j, q, q^(n-1-j)) view, the q entries of a line
           at stride pw[j] */
        const long long inner = pw[j], nlines = N / q;
#pragma omp parallel for schedule(static) num_threads(threads)
        for (long long f = 0; f < nlines; f++) {
            const long long a = f / inner, b = f - a * inner;
            uint8_t *x0 = dist + a * q * inner + b;
            uint8_t m = inf;
            for (int v = 0; v < q; v++) if (x0[v * inner] < m) m = x0[v * inner];
            const uint8_t c = (uint8_t)(m + 1 < inf ? m + 1 : inf);
            for (int v = 0; v < q; v++) if (x0[v * inner] > c) x0[v * inner] = c;
        }
    }
    return 0;
}

int orc_dilate(int q, int n, int R, const uint8_t *code, int M, uint8_t *covered)
{
    long long N = ipw(q, n), pw[32];
    for (int j = 0; j < n; j++) pw[j] = ipw(q, n - 1 - j);
    uint8_t *cur = calloc((size_t)N, 1), *nxt = calloc((size_t)N, 1);
    if (!cur || !nxt) { free(cur); free(nxt); return -1; }
    for (int i = 0; i < M; i++) {
        long long x = 0;
        for (int j = 0; j < n; j++) x += (long long)code[(size_t)i * n + j] * pw[j];
        cur[x] = 1;
    }
    for (int r = 0; r < R; r++) {
        memset(nxt, 0, (size_t)N);
        for (int p = 0; p < n; p++) {
            /* view as (q^p, q, q^(n-1-p)); OR the q entries of every fibre */
            long long outer = ipw(q, p), inner = pw[p];
            for (long long a = 0; a < outer; a++)
                for (long long b = 0; b < inner; b++) {
                    long long x0 = a * q * inner + b;
                    uint8_t any = 0;
                    for (int v = 0; v < q; v++) any |= cur[x0 + (long long)v * inner];
                    if (any)
                        for (int v = 0; v < q; v++) nxt[x0 + (long long)v * inner] = 1;
                }
        }
        uint8_t *t = cur; cur = nxt; nxt = t;
    }
    int all = 1;
    for (long long x = 0; x < N; x++) if (!cur[x]) { all = 0; break; }
    if (covered) memcpy(covered, cur, (size_t)N);
    free(cur); free(nxt);
    return all;
}
