/*
 * covoracle_main.c -- command-line front end of the oracle restatement.
 *
 * TEST INFRASTRUCTURE ONLY.  It speaks the covsearch2e command line
 * (cov/engine/covsearch2e.c:1042-1095) for the flags the p5b path uses and
 * prints the same RESULT line (:1585-1589), so the tests can run the
 * reference binary, this restatement and the GPU engine's CLI on identical
 * arguments and compare fingerprints.  Extra flag: --trace FILE writes one
 * cov_move_rec per move.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "oracle.h"

static const char *DIG = "0123456789abcdefghijklmnopqrstuvwxyz";

static double now_s(void)
{
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* covsearch2e.c:870-898 */
static int read_words(const char *path, int n, uint8_t **out)
{
    FILE *f = fopen(path, "r");
    if (!f) { perror(path); exit(1); }
    char line[4096];
    int m = 0, cap = 1024;
    uint8_t *buf = malloc((size_t)cap * n);
    while (fgets(line, sizeof line, f)) {
        char *h = strchr(line, '#'); if (h) *h = 0;
        uint8_t tmp[64]; int len = 0;
        int spaced = strchr(line, ' ') || strchr(line, ',') || strchr(line, '\t');
        if (spaced) {
            char *tok = strtok(line, " ,\t\r\n");
            while (tok && len < n) { tmp[len++] = (uint8_t)atoi(tok); tok = strtok(NULL, " ,\t\r\n"); }
        } else {
            for (char *s = line; *s && *s != '\n' && *s != '\r'; s++) {
                const char *d = strchr(DIG, *s);
                if (!d || !*d) continue;
                if (len < n) tmp[len++] = (uint8_t)(d - DIG);
            }
        }
        if (len == 0) continue;
        if (len != n) { fprintf(stderr, "%s: bad codeword length %d\n", path, len); exit(1); }
        if (m == cap) { cap *= 2; buf = realloc(buf, (size_t)cap * n); }
        memcpy(buf + (size_t)m * n, tmp, n);
        m++;
    }
    fclose(f);
    *out = buf;
    return m;
}

static void write_words(const char *path, int q, int n, int M, const uint8_t *cw)
{
    uint8_t *buf = malloc((size_t)M * n);
    int m = orc_distinct_code(q, n, M, cw, M, buf);
    char tmp[4096];
    snprintf(tmp, sizeof tmp, "%s.part", path);
    FILE *f = fopen(tmp, "w");
    if (!f) { perror(tmp); free(buf); return; }
    for (int i = 0; i < m; i++) {
        for (int j = 0; j < n; j++) {
            if (q <= 36) fputc(DIG[buf[(size_t)i * n + j]], f);
            else fprintf(f, "%d%s", buf[(size_t)i * n + j], j + 1 < n ? " " : "");
        }
        fputc('\n', f);
    }
    fclose(f);
    rename(tmp, path);
    free(buf);
}

int main(int argc, char **argv)
{
    int q = 0, n = 0, R = -1, M = 0, cand = 100000, tabu = 0, kick = 2, threads = 1;
    int random_init = 0, quiet = 0;
    uint64_t seed = 12345;
    long long iters = -1, stall = 5000, target = -1;
    const char *in = NULL, *out = NULL, *trace = NULL;
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
#define ARG(x) (!strcmp(a, x) && i + 1 < argc)
        if (ARG("-q")) q = atoi(argv[++i]);
        else if (ARG("-n")) n = atoi(argv[++i]);
        else if (ARG("-R")) R = atoi(argv[++i]);
        else if (ARG("-M")) M = atoi(argv[++i]);
        else if (ARG("-t")) ++i;
        else if (ARG("-s")) seed = strtoull(argv[++i], NULL, 10);
        else if (ARG("--in")) in = argv[++i];
        else if (ARG("--out")) out = argv[++i];
        else if (ARG("--cand")) cand = atoi(argv[++i]);
        else if (ARG("--tabu")) tabu = atoi(argv[++i]);
        else if (ARG("--kick")) kick = atoi(argv[++i]);
        else if (ARG("--iters")) iters = atoll(argv[++i]);
        else if (ARG("--stall")) stall = atoll(argv[++i]);
        else if (ARG("--threads")) threads = atoi(argv[++i]);
        else if (ARG("--target")) target = atoll(argv[++i]);
        else if (ARG("--preset")) ++i;
        else if (ARG("--trace")) trace = argv[++i];
        else if (!strcmp(a, "--random-init")) random_init = 1;
        else if (!strcmp(a, "--quiet")) quiet = 1;
        else { fprintf(stderr, "unknown/incomplete option %s\n", a); return 2; }
#undef ARG
    }
    if (q < 2 || n < 1 || R < 0 || M < 1) { fprintf(stderr, "usage: covoracle -q Q -n N -R R -M M ...\n"); return 2; }
    cov_oracle *o = orc_create(q, n, R, M, seed, tabu, kick, stall, cand, threads);
    if (!o) { fprintf(stderr, "bad parameters\n"); return 2; }
    uint8_t *cw = NULL;
    int m = 0;
    if (in) m = read_words(in, n, &cw);
    orc_init(o, cw, m, random_init);
    free(cw);
    if (!quiet) printf("# init uncovered=%lld\n", orc_uncovered(o));
    long long budget = iters >= 0 ? iters : (1LL << 62);
    cov_move_rec *tr = NULL;
    if (trace && iters >= 0) tr = calloc((size_t)(iters > 0 ? iters : 1), sizeof(cov_move_rec));
    double t0 = now_s();
    long long made = (target >= 0 && orc_best_uncovered(o) <= target) ? 0 : orc_run(o, budget, target, tr);
    double el = now_s() - t0;
    printf("RESULT q=%d n=%d R=%d M=%d uncovered=%lld iters=%lld kicks=%lld time=%.2f rate=%.0f\n",
           q, n, R, M, orc_best_uncovered(o), orc_iters(o), orc_kicks(o), el,
           orc_iters(o) / (el > 0 ? el : 1));
    if (tr) {
        FILE *f = fopen(trace, "wb");
        if (f) { fwrite(tr, sizeof(cov_move_rec), (size_t)made, f); fclose(f); }
        free(tr);
    }
    if (out) {
        uint8_t *b = malloc((size_t)M * n);
        orc_get_best(o, b);
        write_words(out, q, n, M, b);
        free(b);
    }
    int rc = orc_best_uncovered(o) == 0 ? 0 : 1;
    orc_destroy(o);
    return rc;
}
