// cov_tiles.cuh -- coverage counting by tiles of the word space, shared by
// the engine's state build (cov_engine.cu) and the verifier's multiplicity
// count (cov_verify.cu).
//
// A tile is the q^nl consecutive words that share their first nh digits.
// Its counters live in shared memory while every codeword within distance R
// of the tile's prefix marks its ball there -- the ball of radius
// R - d(prefix) on the low digits -- so the M*|B| increments of the
// reference's rebuild (covsearch2e.c:958-967, M x ball_apply) are shared-
// memory atomics and the counts reach HBM once.
#pragma once
#include <cstdint>
#include <vector>
#include <algorithm>
#include "cov_common.cuh"

#define BT_MAX 24576           // words of a tile (96 KB of shared memory)
#define BT_LCH 1024            // codewords staged per chunk
#define BT_NT  512             // threads of a tile CTA

// dynamic shared memory of a tile CTA: staged codewords, ids, low indices,
// then the tile's 32-bit counters
static inline size_t bt_smem_bytes(uint32_t tw)
{
    return (size_t)BT_LCH * (8 + 4 + 4) + (size_t)tw * 4;
}

static inline long long bt_ipow(long long b, int e)
{
    long long r = 1;
    while (e-- > 0) r *= b;
    return r;
}

// tile geometry: the most low digits whose q^nl words fit a tile
static inline void bt_geom(int q, int n, int *nh, int *nl)
{
    int l = 1;
    while (l < n && bt_ipow(q, l + 1) <= BT_MAX) l++;
    *nl = l;
    *nh = n - l;
}

// The ball of radius <= min(R, nl) on the low digits nh..n-1 as groups: a
// group fixes the values of the first r-1 positions of an r-subset (nibble
// j of items[] is the value index at position j plus 1, 0 where the centre's
// digit stays) and runs over the q-1 values of its last position last[] (r =
// 0: the centre alone, last = 0xff).  gcum[r] groups have radius <= r.
static inline std::vector<uint64_t> bt_items_h(int q, int n, int R, int nh, uint32_t *gcum,
                                               std::vector<uint8_t> &last)
{
    const int nl = n - nh, rmax = std::min(R, nl);
    std::vector<uint64_t> out;
    last.clear();
    out.push_back(0);
    last.push_back(0xff);
    gcum[0] = 1;
    for (int r = 1; r <= rmax; r++) {
        std::vector<int> sub(r);
        for (int k = 0; k < r; k++) sub[k] = k;
        while (true) {
            std::vector<int> dig(r - 1, 0);
            while (true) {
                uint64_t sp = 0;
                for (int k = 0; k < r - 1; k++) sp |= (uint64_t)(dig[k] + 1) << (4 * (nh + sub[k]));
                out.push_back(sp);
                last.push_back((uint8_t)(nh + sub[r - 1]));
                int k = r - 2;
                while (k >= 0 && dig[k] == q - 2) dig[k--] = 0;
                if (k < 0) break;
                dig[k]++;
            }
            int k = r - 1;
            while (k >= 0 && sub[k] == nl - r + k) k--;
            if (k < 0) break;
            sub[k]++;
            for (int m = k + 1; m < r; m++) sub[m] = sub[m - 1] + 1;
        }
        gcum[r] = (uint32_t)out.size();
    }
    return out;
}

struct BtScratch {
    uint64_t *lpc;             // [BT_LCH] packed codewords of the chunk, grouped by radius
    uint32_t *lid;             // [BT_LCH] their ids
    uint32_t *lbase;           // [BT_LCH] their low-digit word index
    int *gcnt, *gpos, *gfill;  // [COV_MAXN + 2] per radius: count, start, fill
};

// alphabet sizes with their own tile-marking kernels (others run Q = 0)
#define BT_Q_LIST(X) X(5) X(6) X(7) X(8)

// Mark into `tile` (zeroed by the caller) the balls of codewords 0..M-1
// (packed, code[]) intersecting the tile with high digits hp; inc(id) is the
// value added per covered word; items/last/vcum are bt_items_h's groups.
// Q > 0: the alphabet size at compile time (the loop over a group's last
// position unrolled); Q = 0: any q.  Every thread of the CTA (BT_NT) calls it.
template <int Q, class Inc>
__device__ void bt_mark_tile(uint32_t *tile, int q, int n, int R, int M, const uint64_t *__restrict__ code,
                             const uint32_t *pw_in, int nh, int nl, const uint64_t *__restrict__ items,
                             const uint8_t *__restrict__ last, const uint32_t *vcum, uint64_t hp,
                             const BtScratch &sc, Inc inc)
{
    constexpr int PER = BT_LCH / BT_NT;
    // the word strides in shared memory: indexed by position in the inner loop
    __shared__ uint32_t pw[COV_MAXN];
    if (threadIdx.x < COV_MAXN) pw[threadIdx.x] = threadIdx.x < (unsigned)n ? pw_in[threadIdx.x] : 0u;
    __syncthreads();
    const int rmax = min(R, nl);
    const uint64_t hmask = (1ull << (4 * nh)) - 1;   // nh <= 15
    for (int m0 = 0; m0 < M; m0 += BT_LCH) {
        if (threadIdx.x < COV_MAXN + 2) sc.gcnt[threadIdx.x] = 0;
        __syncthreads();
        int g[PER];
        uint64_t pcv[PER];
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int k = m0 + threadIdx.x + u * BT_NT;
            g[u] = -1;
            pcv[u] = 0;
            if (k < M) {
                const uint64_t pc = code[k];
                pcv[u] = pc;
                const int dh = __popcll(cov_spread((pc ^ hp) & hmask));
                if (dh <= R) {
                    g[u] = min(R - dh, nl);
                    atomicAdd(&sc.gcnt[g[u]], 1);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int r = 0; r <= rmax; r++) { sc.gpos[r] = acc; sc.gfill[r] = acc; acc += sc.gcnt[r]; }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PER; u++) {
            if (g[u] < 0) continue;
            const int at = atomicAdd(&sc.gfill[g[u]], 1);
            uint32_t lb = 0;
            for (int j = nh; j < n; j++) lb += (uint32_t)cov_nib(pcv[u], j) * pw[j];
            sc.lpc[at] = pcv[u];
            sc.lid[at] = (uint32_t)(m0 + threadIdx.x + u * BT_NT);
            sc.lbase[at] = lb;
        }
        __syncthreads();
        for (int r = 0; r <= rmax; r++) {
            const uint32_t cnt = (uint32_t)sc.gcnt[r];
            if (!cnt) continue;
            const uint32_t V = vcum[r];
            const uint64_t minv = (0x100000000ull + V - 1) / V;     // ceil(2^32 / V)
            const uint32_t total = cnt * V;
            const int p0 = sc.gpos[r];
            for (uint32_t t = threadIdx.x; t < total; t += BT_NT) {
                uint32_t kk = (uint32_t)(((uint64_t)t * minv) >> 32);   // t / V or one more
                if (kk * V > t) kk--;
                const uint32_t it = t - kk * V;
                const uint64_t pc = sc.lpc[p0 + kk];
                uint64_t sp = items[it];
                int off = (int)sc.lbase[p0 + kk];
                while (sp) {
                    const int j = (__ffsll((long long)sp) - 1) >> 2;
                    const int dig = (int)((sp >> (4 * j)) & 15u) - 1;
                    sp &= ~(15ull << (4 * j));
                    const int cj = cov_nib(pc, j);
                    off += (dig + (dig >= cj) - cj) * (int)pw[j];
                }
                const uint32_t add = inc(sc.lid[p0 + kk]);
                const int lj = last[it];
                if (lj == 0xff) {
                    atomicAdd(&tile[off], add);
                } else {
                    // the q-1 values of the last position other than the centre's
                    const int step = (int)pw[lj];
                    const int cj = cov_nib(pc, lj);
                    int o2 = off - cj * step;
                    if constexpr (Q > 0) {
#pragma unroll
                        for (int v = 0; v < Q; v++, o2 += step)
                            if (v != cj) atomicAdd(&tile[o2], add);
                    } else {
                        for (int v = 0; v < q; v++, o2 += step)
                            if (v != cj) atomicAdd(&tile[o2], add);
                    }
                }
            }
        }
        __syncthreads();
    }
}
