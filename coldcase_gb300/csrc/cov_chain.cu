// cov_chain.cu -- the batched-chains entry point of the reference's GPU
// library, chain_run (cov/gemm2/chainsolve.cu:370-375, bound by
// cov/gemm2/chain.py:30-57), over the pool.
//
// Same arguments and buffers: nchains start codes of M words in rows of 16
// digits, one best code per chain in the same layout, and per chain its best
// uncovered count, whether it covered and the iterations it made.  Each
// chain runs covsearch2e's p5b trajectory (default tenure, kick, stall and
// candidate cap) with search seed seed * 1000003 + chain * 7919 (the
// per-chain seed convention of cov/engine/covengine:557) and stops after
// `iters` moves or when it covers.  `threads` (the reference's CTA size)
// is accepted and not used: the pool sizes its own clusters -- the widest
// power of two (at most 16) with which every chain's cluster is resident at
// once, one CTA per chain when there are more chains than SMs, and one CTA
// for cells too small to share.
#include <cstdio>
#include <vector>
#include <algorithm>
#include "cov_common.cuh"
#include "../../include/covgpu.h"

#define CHAIN_ROW 16            // digits per code row, as chainsolve.cu's MAXN

extern "C" int cov_chain_run(int q, int n, int R, int M, int nchains, long long iters, unsigned long long seed,
                             int threads, const uint8_t *code_h, uint8_t *best_h, int32_t *best_u_h,
                             int32_t *solved_h, long long *iters_h)
{
    (void)threads;
    if (q < 2 || q > 16 || n < 1 || n > CHAIN_ROW || R < 0 || M < 1 || nchains < 1 || iters < 0 || !code_h ||
        !best_h || !best_u_h || !solved_h || !iters_h)
        return COV_EINVAL;
    long long N = 1;
    for (int j = 0; j < n; j++) N *= q;
    int cluster = 1;
    const int sms = std::max(1, cov_sm_count());
    while (N >= (1LL << 16) && cluster < 16 && (long long)nchains * cluster * 2 <= sms) cluster *= 2;
    cov_pool *pool = nullptr;
    int rc = cov_pool_create(nchains, cluster, &pool);
    if (rc) return rc;
    rc = cov_pool_set_budget(pool, 60.0);
    std::vector<int32_t> slot(nchains, -1);
    std::vector<uint8_t> code((size_t)M * n);
    for (int c = 0; c < nchains && !rc; c++) {
        for (int i = 0; i < M; i++)
            for (int j = 0; j < n; j++) {
                const uint8_t v = code_h[((size_t)c * M + i) * CHAIN_ROW + j];
                if (v >= q) { rc = COV_EINVAL; break; }
                code[(size_t)i * n + j] = v;
            }
        if (rc) break;
        cov_params prm = {};
        prm.q = q; prm.n = n; prm.R = R; prm.M = M;
        prm.seed = seed * 1000003ull + (unsigned long long)c * 7919ull;
        prm.tabu = 0; prm.kick = 2; prm.cand = 100000; prm.stall = 5000;
        rc = cov_pool_add(pool, &prm, code.data(), M, 0, &slot[c]);
        if (!rc) rc = cov_pool_set_slot_param(pool, slot[c], "it_limit", iters);
    }
    // run to the iteration limits; a launch that reaches its wall-clock
    // budget stops its slots between moves, and they resume where they were
    std::vector<cov_status> st(nchains);
    for (int round = 0; !rc && round < 1000000; round++) {
        rc = cov_pool_run(pool, iters, -1);
        if (rc) break;
        bool more = false;
        for (int c = 0; c < nchains && !rc; c++) {
            rc = cov_pool_status(pool, slot[c], &st[c]);
            if (rc) break;
            if (st[c].status == COV_ETIMEOUT) {
                rc = cov_pool_resume(pool, slot[c]);
                more = true;
            } else if (st[c].status != 0) {
                rc = st[c].status;
            } else if (st[c].it < iters && !st[c].finished) {
                more = true;
            }
        }
        if (!more) break;
    }
    for (int c = 0; c < nchains && !rc; c++) {
        rc = cov_pool_get_best(pool, slot[c], code.data());
        if (rc) break;
        uint8_t *row = best_h + (size_t)c * M * CHAIN_ROW;
        std::fill(row, row + (size_t)M * CHAIN_ROW, (uint8_t)0);
        for (int i = 0; i < M; i++)
            for (int j = 0; j < n; j++) row[(size_t)i * CHAIN_ROW + j] = code[(size_t)i * n + j];
        best_u_h[c] = (int32_t)st[c].best;
        solved_h[c] = st[c].best == 0;
        iters_h[c] = st[c].it;
    }
    const int rd = cov_pool_destroy(pool);
    return rc ? rc : rd;
}
