// cov_lns.cu -- GB300 (sm_103a) transform engine for the ruin-and-recreate
// search over one cell (q, n, R): the capability of cov/gemm2/gpuchain.py
// and its primitives cov/gemm2/dct.cu, built around two device-side pieces.
//
//  * Maps.  gain(x) = #{y : d(x,y) <= R, cnt[y] == 0} (the words a codeword
//    at x would newly cover) and loss(x) = the same with cnt[y] == 1 (the
//    words only a codeword at x covers) are computed for every x at once as
//    layered counts: L_d[x] = #{marked y : d(x,y) = d}, d = 0..R, built one
//    axis at a time -- along a line of q words with layer sums S_d, a word's
//    L_d gains S_{d-1} - L_{d-1}[x] (the marked words that now differ from it
//    in this coordinate too) -- and summed over d at the end.  The axes are
//    not swept one by one through HBM: the low axes are done on contiguous
//    tiles of q^k words in shared memory, the remaining ones on strips of
//    q^g rows x W words, all R+1 int32 layers of a tile at once, so a whole
//    transform reads and writes the layers in a few sweeps instead of n.
//    The same layers with the code itself marked give cnt.
//  * Sequences.  A persistent kernel on one thread-block cluster runs the
//    steps that are inherently one after another, with no host round trip:
//    the lazy greedy placement (bounds from a gain map, the best bound
//    re-counted exactly until it is current, then placed), the exact peel
//    (codewords removed in a given order while each covers no word alone)
//    and +-1 balls of a list of words.  Every CTA of the cluster walks a
//    share of each ball; they meet at hardware cluster barriers and reduce
//    through distributed shared memory.
//
// Words are indexed MSB-first (x = sum_j w_j q^(n-1-j)), as everywhere in
// this library.  Extraction returns positions in increasing index order, and
// every tie is broken by the lower position, so every result is
// deterministic.
#include <cstdio>
#include <climits>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cooperative_groups.h>
#include "cov_common.cuh"
#include "cov_tiles.cuh"
#include "../../include/covgpu.h"

namespace cg = cooperative_groups;

#define LNS_MAXR 8
#define LNS_NT 256
#define LNS_HIST_MAX 8192   // bins of cov_lns_map_hist (one shared-memory counter each)
#define MAP_NT 512
#define MAP_SMEM_MAX (200 * 1024)   // shared memory of one map tile (bytes)
#define MAP_W_MIN 8                 // narrowest strip: 32 bytes of a layer per row
#define SEQ_NT 512
#define SEQ_CL 8                    // CTAs of the sequence cluster
#define CAND_CAP (1 << 17)          // candidate bounds kept on the device per refresh

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "covgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    return -(100 + (int)e_); } } while (0)

// state of a sequence launch, read back by the host
struct SeqState {
    long long uncov;             // uncovered words, kept exact through every ball
    long long evals;             // exact ball counts made
    int placed, removed;         // words placed / removed by the launch
    int status;                  // SEQ_*
    int pad;
};
enum { SEQ_DONE = 0, SEQ_REFRESH = 1, SEQ_COVERED = 2, SEQ_TARGET = 3, SEQ_GUARD = 5 };
enum { MODE_GREEDY = 0, MODE_PEEL = 1, MODE_APPLY = 2 };

struct cov_lns {
    int q, n, R;
    uint32_t N;
    uint32_t pw[COV_MAXN];          // q^(n-1-j)
    uint16_t *cnt = nullptr;        // coverage multiplicity (saturated)
    int32_t *layer[LNS_MAXR + 1] = {};
    int32_t *map = nullptr;         // last map (gain or loss)
    uint64_t *ball = nullptr;       // whole-ball groups (cov_tiles.cuh, no high digits)
    uint8_t *ball_last = nullptr;
    uint32_t ngroups = 0;
    uint32_t *cand = nullptr;       // greedy candidates (positions, increasing)
    int32_t *bound = nullptr;       // their gain bounds
    int32_t *fresh = nullptr;       // epoch at which a bound was last made exact
    uint32_t *list = nullptr;       // words of a sequence (placed, peeled or applied)
    uint8_t *flag = nullptr;        // per listed word: removed by the peel
    SeqState *seq = nullptr;
    void *scratch = nullptr;        // small device buffers of the calls
    size_t scratch_bytes = 0;
    unsigned long long *d_red = nullptr;
};

namespace {

struct LayerPtrs { int32_t *a[LNS_MAXR + 1]; };

struct MapGeom {
    int q, n;
    uint32_t N;
    uint32_t pk[COV_MAXN + 1];      // q^k: the stride of axis k (the digit n-1-k)
};

// ----------------------------------------------------------- the maps -----
// One axis over `nfib` lines of q elements at element stride st, held in
// shared memory as R1 layers of E elements each.  Each thread owns whole
// lines, so the update needs no synchronisation inside a pass.  With the
// alphabet size Q known at compile time a line's Q x R1 counts are read
// once into registers (R1 loads and R1 - 1 stores per element, no division
// by st); Q = 0 is the form for any q.
template <int R1, int Q>
__device__ __forceinline__ void map_axis(int32_t *Ls, uint32_t E, int q, uint32_t nfib, uint32_t st)
{
    if constexpr (Q > 0) {
        // f / st by a float reciprocal: f < 2^24, so the estimate is off by
        // at most one and one correction makes it exact
        const float rinv = 1.0f / (float)st;
        for (uint32_t f = threadIdx.x; f < nfib; f += blockDim.x) {
            int o = (int)((float)f * rinv);
            int i = (int)f - o * (int)st;
            if (i < 0) { o--; i += (int)st; } else if (i >= (int)st) { o++; i -= (int)st; }
            const uint32_t e0 = (uint32_t)o * st * (uint32_t)Q + (uint32_t)i;
            int32_t v[Q][R1];
#pragma unroll
            for (int a = 0; a < Q; a++)
#pragma unroll
                for (int d = 0; d < R1; d++) v[a][d] = Ls[d * E + e0 + (uint32_t)a * st];
            int32_t S[R1 > 1 ? R1 - 1 : 1];
#pragma unroll
            for (int d = 0; d < R1 - 1; d++) {
                S[d] = 0;
#pragma unroll
                for (int a = 0; a < Q; a++) S[d] += v[a][d];
            }
#pragma unroll
            for (int a = 0; a < Q; a++)
#pragma unroll
                for (int d = 1; d < R1; d++) Ls[d * E + e0 + (uint32_t)a * st] = v[a][d] + S[d - 1] - v[a][d - 1];
        }
        return;
    }
    for (uint32_t f = threadIdx.x; f < nfib; f += blockDim.x) {
        const uint32_t o = f / st, i = f - o * st;
        const uint32_t e0 = o * st * (uint32_t)q + i;
        int32_t S[R1 > 1 ? R1 - 1 : 1];
#pragma unroll
        for (int d = 0; d < R1 - 1; d++) S[d] = 0;
        for (int a = 0; a < q; a++) {
            const uint32_t e = e0 + (uint32_t)a * st;
#pragma unroll
            for (int d = 0; d < R1 - 1; d++) S[d] += Ls[d * E + e];
        }
        for (int a = 0; a < q; a++) {
            const uint32_t e = e0 + (uint32_t)a * st;
            int32_t below = Ls[e];                    // old L_{d-1}[x], starting at L_0
#pragma unroll
            for (int d = 1; d < R1; d++) {
                const int32_t old = Ls[d * E + e];
                Ls[d * E + e] = old + S[d - 1] - below;
                below = old;
            }
        }
    }
}

template <int R1>
__device__ __forceinline__ void map_out(int32_t *Ls, uint32_t E, uint32_t e, uint32_t x, int fin, LayerPtrs L,
                                        int32_t *out, uint16_t *cnt16)
{
    if (fin) {
        int32_t s = 0;
#pragma unroll
        for (int d = 0; d < R1; d++) s += Ls[d * E + e];
        if (out) out[x] = s;
        else cnt16[x] = (uint16_t)min(s, 65535);
    } else {
#pragma unroll
        for (int d = 0; d < R1; d++) L.a[d][x] = Ls[d * E + e];
    }
}

// Axes 0..k-1 on contiguous tiles of T = q^k words.  Layer 0 starts as
// [cnt == target] (cnt given) or as the layer-0 array (the code's word
// counts); the higher layers start at 0.  With fin (k == n) the map is
// written, else the layers.
template <int R1, int Q>
__global__ void __launch_bounds__(MAP_NT) k_map_low(MapGeom g, int k, const uint16_t *__restrict__ cnt, int target,
                                                    LayerPtrs L, int fin, int32_t *out, uint16_t *cnt16)
{
    extern __shared__ __align__(16) int32_t Ls[];
    uint32_t T = 1;
    for (int j = 0; j < k; j++) T *= (uint32_t)g.q;
    const uint32_t ntile = g.N / T;
    for (uint32_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const uint32_t x0 = tile * T;
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < T; e += blockDim.x) {
            const uint32_t x = x0 + e;
            Ls[e] = cnt ? (int32_t)(__ldcg(&cnt[x]) == target) : L.a[0][x];
#pragma unroll
            for (int d = 1; d < R1; d++) Ls[d * T + e] = 0;
        }
        __syncthreads();
        uint32_t st = 1;
        for (int j = 0; j < k; j++, st *= (uint32_t)g.q) {
            map_axis<R1, Q>(Ls, T, g.q, T / (uint32_t)g.q, st);
            __syncthreads();
        }
        for (uint32_t e = threadIdx.x; e < T; e += blockDim.x) map_out<R1>(Ls, T, e, x0 + e, fin, L, out, cnt16);
    }
}

// Axes j0..j0+gsz-1 on strips: q^gsz rows (row r at stride s = q^j0) of
// W = 2^lw consecutive words, element (r, c) at base + r*s + c.
template <int R1, int Q>
__global__ void __launch_bounds__(MAP_NT) k_map_high(MapGeom g, int j0, int gsz, int lw, LayerPtrs L, int fin,
                                                     int32_t *out, uint16_t *cnt16)
{
    extern __shared__ __align__(16) int32_t Ls[];
    const uint32_t W = 1u << lw;
    uint32_t s = 1, rows = 1;
    for (int j = 0; j < j0; j++) s *= (uint32_t)g.q;
    for (int j = 0; j < gsz; j++) rows *= (uint32_t)g.q;
    const uint32_t E = rows << lw;
    const uint32_t span = rows * s, outer = g.N / span;
    const uint32_t nstrip = (s + W - 1) >> lw;
    const unsigned long long ntiles = (unsigned long long)outer * nstrip;
    for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t o = (uint32_t)(tile / nstrip);
        const uint32_t c0 = (uint32_t)(tile - (unsigned long long)o * nstrip) << lw;
        const uint32_t w = min(W, s - c0);
        const uint32_t base = o * span + c0;
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < E; e += blockDim.x) {
            const uint32_t r = e >> lw, c = e & (W - 1);
            const uint32_t x = base + r * s + c;
#pragma unroll
            for (int d = 0; d < R1; d++) Ls[d * E + e] = c < w ? L.a[d][x] : 0;
        }
        __syncthreads();
        uint32_t st = W;
        for (int jj = 0; jj < gsz; jj++, st *= (uint32_t)g.q) {
            map_axis<R1, Q>(Ls, E, g.q, E / (uint32_t)g.q, st);
            __syncthreads();
        }
        for (uint32_t e = threadIdx.x; e < E; e += blockDim.x) {
            const uint32_t r = e >> lw, c = e & (W - 1);
            if (c < w) map_out<R1>(Ls, E, e, base + r * s + c, fin, L, out, cnt16);
        }
    }
}

__global__ void k_lns_zero_layer(int32_t *A0, uint32_t N)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) A0[x] = 0;
}

__global__ void k_lns_scatter(int32_t *A0, const uint32_t *idx, int m)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) atomicAdd(&A0[idx[i]], 1);
}

// R = 0: the map is the indicator itself
__global__ void k_lns_indicator(const uint16_t *cnt, int target, const int32_t *A0, uint32_t N, int32_t *out,
                                uint16_t *cnt16)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) {
        const int32_t v = cnt ? (int32_t)(cnt[x] == target) : A0[x];
        if (out) out[x] = v;
        else cnt16[x] = (uint16_t)min(v, 65535);
    }
}

__global__ void k_lns_max(const int32_t *A, uint32_t N, int *out)
{
    int m = INT_MIN;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) m = max(m, A[x]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// histogram of values v >= 1 in nbins bins of [1, vmax]: bin = (v-1)*nbins/vmax
// histogram of the positive values: value v in bin (min(v,vmax)-1)*nbins/vmax.
// Counted per block in shared memory (the lanes of a warp that share a bin
// add once), then one global add per bin and block: the values of a gain map
// crowd into few bins, where per-element global atomics serialise.
__global__ void k_lns_hist(const int32_t *A, uint32_t N, int nbins, int vmax, unsigned long long *hist)
{
    extern __shared__ uint32_t lh[];
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) lh[b] = 0;
    __syncthreads();
    // (v-1)*nbins in 32 bits when it cannot overflow
    const bool narrow = (unsigned long long)vmax * (unsigned long long)nbins < (1ull << 32);
    for (uint32_t x0 = blockIdx.x * blockDim.x; x0 < N; x0 += gridDim.x * blockDim.x) {
        const uint32_t x = x0 + threadIdx.x;
        int b = -1;
        if (x < N) {
            const int v = A[x];
            if (v >= 1) {
                const uint32_t t = (uint32_t)(min(v, vmax) - 1);
                b = narrow ? (int)(t * (uint32_t)nbins / (uint32_t)vmax)
                           : (int)((unsigned long long)t * (unsigned long long)nbins / (unsigned long long)vmax);
            }
        }
        const unsigned grp = __match_any_sync(0xffffffffu, b);
        if (b >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&lh[b], (uint32_t)__popc(grp));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
        if (lh[b]) atomicAdd(&hist[b], (unsigned long long)lh[b]);
}

// ordered compaction of {x : A[x] >= thr}: per-block counts, then positions
__global__ void k_lns_count_ge(const int32_t *A, uint32_t N, int thr, uint32_t chunk, uint32_t *bcount)
{
    const uint32_t x0 = blockIdx.x * chunk, x1 = min(N, x0 + chunk);
    uint32_t c = 0;
    for (uint32_t x = x0 + threadIdx.x; x < x1; x += blockDim.x) c += A[x] >= thr;
    __shared__ uint32_t red[LNS_NT / 32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < LNS_NT / 32; w++) s += red[w];
        bcount[blockIdx.x] = s;
    }
}

__global__ void k_lns_emit_ge(const int32_t *A, uint32_t N, int thr, uint32_t chunk, const uint32_t *boff,
                              uint32_t cap, uint32_t *oidx, int32_t *oval)
{
    const uint32_t x0 = blockIdx.x * chunk, x1 = min(N, x0 + chunk);
    __shared__ uint32_t wbase[LNS_NT / 32];
    __shared__ uint32_t run;
    if (threadIdx.x == 0) run = boff[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t xb = x0; xb < x1; xb += blockDim.x) {
        const uint32_t x = xb + threadIdx.x;
        const bool take = x < x1 && A[x] >= thr;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (lane == 0) wbase[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t s = run;
            for (int w = 0; w < LNS_NT / 32; w++) { const uint32_t c = wbase[w]; wbase[w] = s; s += c; }
            run = s;
        }
        __syncthreads();
        if (take) {
            const uint32_t at = wbase[warp] + __popc(m & ((1u << lane) - 1));
            if (at < cap) { oidx[at] = x; oval[at] = A[x]; }
        }
        __syncthreads();
    }
}

// decode a packed word from its index
__device__ __forceinline__ uint64_t lns_pack(uint32_t x, int q, int n)
{
    uint64_t pk = 0;
    for (int j = n - 1; j >= 0; j--) { pk |= (uint64_t)(x % (uint32_t)q) << (4 * j); x /= (uint32_t)q; }
    return pk;
}

struct BallGeom {
    int q, n;
    uint32_t pw[COV_MAXN];
    const uint64_t *items;
    const uint8_t *last;
    uint32_t ngroups;
};

// The words of ball group `it` of the ball around base (packed pc): calls
// f(word) for each (one word, or the q-1 values of the group's last position).
template <class F>
__device__ __forceinline__ void ball_group(const BallGeom &b, uint32_t it, uint32_t base, uint64_t pc, F f)
{
    uint64_t sp = b.items[it];
    int off = (int)base;
    while (sp) {
        const int j = (__ffsll((long long)sp) - 1) >> 2;
        const int dig = (int)((sp >> (4 * j)) & 15u) - 1;
        sp &= ~(15ull << (4 * j));
        const int cj = cov_nib(pc, j);
        off += (dig + (dig >= cj) - cj) * (int)b.pw[j];
    }
    const int lj = b.last[it];
    if (lj == 0xff) {
        f((uint32_t)off);
    } else {
        const int step = (int)b.pw[lj], cj = cov_nib(pc, lj);
        int o2 = off - cj * step;
        for (int v = 0; v < b.q; v++, o2 += step)
            if (v != cj) f((uint32_t)o2);
    }
}

// One CTA per listed word: #{y in its ball : cnt[y] == target} (the
// independent exact counts of many words at once).
__global__ void k_lns_gather(const uint16_t *cnt, const uint32_t *idx, int k, BallGeom b, int target, int32_t *out)
{
    const int i = blockIdx.x;
    if (i >= k) return;
    const uint32_t base = idx[i];
    const uint64_t pc = lns_pack(base, b.q, b.n);
    int c = 0;
    for (uint32_t it = threadIdx.x; it < b.ngroups; it += blockDim.x)
        ball_group(b, it, base, pc, [&](uint32_t w) { c += __ldcg(&cnt[w]) == target; });
    __shared__ int red[32];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) s += red[w];
        out[i] = s;
    }
}

__global__ void k_lns_read(const int32_t *A, const uint32_t *idx, int k, int32_t *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) out[i] = A[idx[i]];
}

__global__ void k_lns_zero(const uint16_t *cnt, uint32_t N, int target, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        c += cnt[x] == target;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ------------------------------------------------------- the sequences ----
struct SeqArgs {
    int mode;
    uint16_t *cnt;
    BallGeom b;
    // greedy: candidates (increasing positions) and their bounds; placed
    // words are appended to list[]
    const uint32_t *cand;
    int32_t *bound;
    int32_t *fresh;
    int ncand, thr, room;          // room: words still to place
    int eval_cap;                  // exact counts since the last placement after which a
                                   // fresh map is cheaper (the host refreshes)
    long long max_steps;           // bound on the steps of one launch
    // peel / apply: the listed words in order
    uint32_t *list;
    int nlist, sign;
    uint8_t *flag;
    SeqState *st;
};

struct SeqShared {
    unsigned long long cbest[SEQ_CL];  // greedy: each CTA's max key (plain stores, one per CTA)
    long long sum;                 // ball count / crossings over the cluster
    int act, pos;                  // the leader's decision
    uint32_t word;
    int stop;
};

// a ball walked by the whole cluster: count (op 0: cnt == target) or add
// sgn (op 1; returns the words that crossed between 0 and 1, signed as the
// uncovered count changes).  All words of one ball are distinct.
__device__ __forceinline__ long long cluster_ball(const SeqArgs &a, uint32_t base, int op, int target, int sgn,
                                                  int rank)
{
    const uint64_t pc = lns_pack(base, a.b.q, a.b.n);
    long long c = 0;
    for (uint32_t it = (uint32_t)rank * SEQ_NT + threadIdx.x; it < a.b.ngroups; it += SEQ_CL * SEQ_NT) {
        ball_group(a.b, it, base, pc, [&](uint32_t w) {
            const uint32_t v = __ldcg(&a.cnt[w]);
            if (op == 0) {
                c += v == (uint32_t)target;
            } else if (sgn > 0) {
                if (v != 65535u) __stcg(&a.cnt[w], (uint16_t)(v + 1));
                c -= v == 0;                          // newly covered
            } else {
                if (v != 0u) __stcg(&a.cnt[w], (uint16_t)(v - 1));
                c += v == 1;                          // newly uncovered
            }
        });
    }
    return c;
}

// reduce a per-thread value into the leader CTA's shared sum
__device__ __forceinline__ void cluster_add(long long v, SeqShared *lead)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long *)&lead->sum, (unsigned long long)v);
}

enum { ACT_STOP = 0, ACT_EVAL, ACT_PLACE, ACT_NEXT };

// key of a candidate: larger bound first, then the lower position
__device__ __forceinline__ unsigned long long cand_key(int32_t bound, int pos)
{
    return ((unsigned long long)(uint32_t)(bound + 0x40000000) << 32) | (uint32_t)(0x7fffffff - pos);
}

__global__ void __cluster_dims__(SEQ_CL, 1, 1) __launch_bounds__(SEQ_NT) k_lns_seq(SeqArgs a)
{
    __shared__ SeqShared sh;
    __shared__ unsigned long long s_wmax[SEQ_NT / 32];
    __shared__ long long s_uncov, s_evals, s_steps;
    __shared__ int s_epoch, s_placed, s_removed, s_i, s_since;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    SeqShared *lead = cl.map_shared_rank(&sh, 0);
    if (threadIdx.x == 0) {
        for (int r = 0; r < SEQ_CL; r++) sh.cbest[r] = 0;
        sh.sum = 0; sh.act = ACT_NEXT; sh.stop = 0; sh.pos = 0; sh.word = 0;
        if (rank == 0) {
            s_uncov = a.st->uncov; s_evals = 0; s_steps = 0;
            s_epoch = 1; s_placed = 0; s_removed = 0; s_i = 0; s_since = 0;
        }
    }
    __syncthreads();
    cl.sync();
    for (;;) {
        // ---- the leader decides the next step
        if (a.mode == MODE_GREEDY) {
            unsigned long long k = 0;
            for (int p = rank * SEQ_NT + threadIdx.x; p < a.ncand; p += SEQ_CL * SEQ_NT)
                k = max(k, cand_key(__ldcg(&a.bound[p]), p));
            for (int o = 16; o > 0; o >>= 1) k = max(k, __shfl_xor_sync(0xffffffffu, k, o));
            if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = k;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long kc = 0;
                for (int w = 0; w < SEQ_NT / 32; w++) kc = max(kc, s_wmax[w]);
                lead->cbest[rank] = kc;
            }
            cl.sync();
            if (rank == 0 && threadIdx.x == 0) {
                unsigned long long k0 = 0;
                for (int r = 0; r < SEQ_CL; r++) k0 = max(k0, sh.cbest[r]);
                const int pos = k0 ? 0x7fffffff - (int)(uint32_t)k0 : -1;
                const int bnd = k0 ? (int)(uint32_t)(k0 >> 32) - 0x40000000 : 0;
                int st = -1;
                if (s_uncov <= 0) st = SEQ_COVERED;
                else if (s_placed >= a.room) st = SEQ_TARGET;
                else if (++s_steps > a.max_steps) st = SEQ_GUARD;
                // below the threshold a word outside the candidates could tie
                // or beat the best: the host refreshes the bounds (and stops
                // when the fresh map has no positive gain)
                else if (pos < 0 || bnd < a.thr) st = SEQ_REFRESH;
                // so many bounds went stale that a fresh map is cheaper
                else if (s_since >= a.eval_cap && __ldcg(&a.fresh[pos]) != s_epoch) st = SEQ_REFRESH;
                if (st >= 0) {
                    sh.act = ACT_STOP;
                    a.st->status = st;
                } else if (__ldcg(&a.fresh[pos]) == s_epoch) {
                    // exact, and no other bound is higher: the best placement
                    sh.act = ACT_PLACE; sh.pos = pos; sh.word = a.cand[pos];
                } else {
                    sh.act = ACT_EVAL; sh.pos = pos; sh.word = a.cand[pos];
                }
                sh.sum = 0;
            }
        } else {
            // every CTA has read the previous step's decision before the
            // leader writes the next one
            cl.sync();
            if (rank == 0 && threadIdx.x == 0) {
                if (s_i >= a.nlist || ++s_steps > a.max_steps) {
                    sh.act = ACT_STOP;
                    a.st->status = s_i >= a.nlist ? SEQ_DONE : SEQ_GUARD;
                } else {
                    sh.act = a.mode == MODE_PEEL ? ACT_EVAL : ACT_PLACE;
                    sh.pos = s_i; sh.word = a.list[s_i];
                }
                sh.sum = 0;
            }
        }
        cl.sync();
        const int act = lead->act;
        const int pos = lead->pos;
        const uint32_t word = lead->word;
        if (act == ACT_STOP) break;
        // ---- the step on the whole cluster
        if (act == ACT_EVAL) {
            // greedy: the exact gain (count of uncovered ball words);
            // peel: the exact loss (count of ball words covered only once)
            cluster_add(cluster_ball(a, word, 0, a.mode == MODE_GREEDY ? 0 : 1, 0, rank), lead);
            cl.sync();
            if (rank == 0 && threadIdx.x == 0) {
                s_evals++;
                if (a.mode == MODE_GREEDY) {
                    __stcg(&a.bound[pos], (int32_t)sh.sum);
                    __stcg(&a.fresh[pos], s_epoch);
                    s_since++;
                    sh.act = ACT_NEXT;
                } else {
                    sh.act = sh.sum == 0 ? ACT_PLACE : ACT_NEXT;    // peel: remove if it covers nothing alone
                    if (sh.act == ACT_NEXT) s_i++;
                }
                sh.sum = 0;
            }
            cl.sync();
            if (a.mode == MODE_GREEDY || lead->act != ACT_PLACE) continue;
        }
        // place (greedy, apply +1) or remove (peel, apply -1) the word's ball
        const int sgn = a.mode == MODE_GREEDY ? 1 : a.mode == MODE_PEEL ? -1 : a.sign;
        cluster_add(cluster_ball(a, word, 1, 0, sgn, rank), lead);
        cl.sync();
        if (rank == 0 && threadIdx.x == 0) {
            s_uncov += sh.sum;
            sh.sum = 0;
            if (a.mode == MODE_GREEDY) {
                a.list[s_placed++] = word;
                __stcg(&a.bound[pos], 0);         // a codeword now: its ball is covered
                s_epoch++;
                s_since = 0;
            } else {
                if (a.mode == MODE_PEEL) { a.flag[s_i] = 1; s_removed++; }
                s_i++;
            }
        }
        cl.sync();
    }
    if (rank == 0 && threadIdx.x == 0) {
        a.st->uncov = s_uncov;
        a.st->evals = s_evals;
        a.st->placed = s_placed;
        a.st->removed = s_removed;
    }
    // no CTA may leave while another can still reach the leader's shared memory
    cl.sync();
}

int grid_of(uint32_t N)
{
    return (int)std::min<uint32_t>((N + LNS_NT - 1) / LNS_NT, (uint32_t)std::max(1, cov_sm_count()) * 8);
}

CovDeviceFlags g_map_attr;      // shared-memory opt-in of the map kernels, per device

// alphabet sizes with their own map kernels (others run the Q = 0 form)
#define MAP_Q_LIST(X) X(5) X(6) X(7) X(8)

template <int R1, int Q>
int map_attrs_rq()
{
    CK(cudaFuncSetAttribute(k_map_low<R1, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, MAP_SMEM_MAX));
    CK(cudaFuncSetAttribute(k_map_high<R1, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, MAP_SMEM_MAX));
    return 0;
}

template <int R1>
int map_attrs_one()
{
    int rc = map_attrs_rq<R1, 0>();
#define MAP_ATTR_Q(QQ) if (!rc) rc = map_attrs_rq<R1, QQ>();
    MAP_Q_LIST(MAP_ATTR_Q)
#undef MAP_ATTR_Q
    return rc;
}

int map_attrs()
{
    int dev = 0;
    if (g_map_attr.done(dev)) return 0;
    int rc = map_attrs_one<2>();
    if (!rc) rc = map_attrs_one<3>();
    if (!rc) rc = map_attrs_one<4>();
    if (!rc) rc = map_attrs_one<5>();
    if (!rc) rc = map_attrs_one<6>();
    if (!rc) rc = map_attrs_one<7>();
    if (!rc) rc = map_attrs_one<8>();
    if (!rc) rc = map_attrs_one<9>();
    if (rc) return rc;
    g_map_attr.set(dev);
    return 0;
}

template <int R1>
int map_launch_low(int grid, size_t smem, const MapGeom &g, int k, const uint16_t *cnt, int target, LayerPtrs L,
                   int fin, int32_t *out, uint16_t *cnt16)
{
    switch (g.q) {
#define MAP_LOW_Q(QQ) case QQ: k_map_low<R1, QQ><<<grid, MAP_NT, smem>>>(g, k, cnt, target, L, fin, out, cnt16); break;
    MAP_Q_LIST(MAP_LOW_Q)
#undef MAP_LOW_Q
    default: k_map_low<R1, 0><<<grid, MAP_NT, smem>>>(g, k, cnt, target, L, fin, out, cnt16); break;
    }
    CK(cudaGetLastError());
    return 0;
}

template <int R1>
int map_launch_high(int grid, size_t smem, const MapGeom &g, int j0, int gsz, int lw, LayerPtrs L, int fin,
                    int32_t *out, uint16_t *cnt16)
{
    switch (g.q) {
#define MAP_HIGH_Q(QQ) case QQ: k_map_high<R1, QQ><<<grid, MAP_NT, smem>>>(g, j0, gsz, lw, L, fin, out, cnt16); break;
    MAP_Q_LIST(MAP_HIGH_Q)
#undef MAP_HIGH_Q
    default: k_map_high<R1, 0><<<grid, MAP_NT, smem>>>(g, j0, gsz, lw, L, fin, out, cnt16); break;
    }
    CK(cudaGetLastError());
    return 0;
}

int map_low_any(int R1, int grid, size_t smem, const MapGeom &g, int k, const uint16_t *cnt, int target,
                LayerPtrs L, int fin, int32_t *out, uint16_t *cnt16)
{
    switch (R1) {
    case 2: return map_launch_low<2>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 3: return map_launch_low<3>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 4: return map_launch_low<4>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 5: return map_launch_low<5>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 6: return map_launch_low<6>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 7: return map_launch_low<7>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 8: return map_launch_low<8>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    case 9: return map_launch_low<9>(grid, smem, g, k, cnt, target, L, fin, out, cnt16);
    default: return COV_EINVAL;
    }
}

int map_high_any(int R1, int grid, size_t smem, const MapGeom &g, int j0, int gsz, int lw, LayerPtrs L, int fin,
                 int32_t *out, uint16_t *cnt16)
{
    switch (R1) {
    case 2: return map_launch_high<2>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 3: return map_launch_high<3>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 4: return map_launch_high<4>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 5: return map_launch_high<5>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 6: return map_launch_high<6>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 7: return map_launch_high<7>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 8: return map_launch_high<8>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    case 9: return map_launch_high<9>(grid, smem, g, j0, gsz, lw, L, fin, out, cnt16);
    default: return COV_EINVAL;
    }
}

// The layered transform: layer 0 from [cnt == target] (cnt given) or from
// the layer-0 array (the code's counts), result to out (int32 map) or cnt16.
int lns_transform(cov_lns *h, const uint16_t *cnt, int target, int32_t *out, uint16_t *cnt16)
{
    LayerPtrs L;
    for (int d = 0; d <= LNS_MAXR; d++) L.a[d] = d <= h->R ? h->layer[d] : nullptr;
    if (h->R == 0) {
        k_lns_indicator<<<grid_of(h->N), LNS_NT>>>(cnt, target, h->layer[0], h->N, out, cnt16);
        CK(cudaGetLastError());
        return 0;
    }
    int rc = map_attrs();
    if (rc) return rc;
    const int R1 = h->R + 1, q = h->q, n = h->n;
    MapGeom g;
    memset(&g, 0, sizeof g);
    g.q = q; g.n = n; g.N = h->N;
    g.pk[0] = 1;
    for (int k = 1; k <= n; k++) g.pk[k] = g.pk[k - 1] * (uint32_t)q;
    const size_t per = (size_t)R1 * 4;                    // bytes of one element's layers
    const int sms = std::max(1, cov_sm_count());
    // low axes: the widest contiguous tile the shared memory holds
    int k = 1;
    while (k < n && (size_t)g.pk[k + 1] * per <= MAP_SMEM_MAX) k++;
    if ((size_t)g.pk[k] * per > MAP_SMEM_MAX) return COV_ERANGE;
    {
        const size_t smem = (size_t)g.pk[k] * per;
        const int per_sm = std::max(1, (int)(220 * 1024 / smem));
        const int grid = (int)std::min<uint32_t>(h->N / g.pk[k], (uint32_t)(sms * per_sm));
        rc = map_low_any(R1, grid, smem, g, k, cnt, target, L, k == n, out, cnt16);
        if (rc) return rc;
    }
    // the other axes in strips: as many axes as fit with rows of at least
    // MAP_W_MIN words, then as wide as the shared memory allows
    int j0 = k;
    while (j0 < n) {
        int gsz = 0;
        while (j0 + gsz < n && (size_t)g.pk[gsz + 1] * MAP_W_MIN * per <= MAP_SMEM_MAX) gsz++;
        if (gsz == 0) return COV_ERANGE;
        const uint32_t s = g.pk[j0];
        int lw = 0;
        while ((size_t)g.pk[gsz] * ((size_t)2 << lw) * per <= MAP_SMEM_MAX && (1u << lw) < s) lw++;
        const size_t smem = ((size_t)g.pk[gsz] << lw) * per;
        const unsigned long long tiles =
            (unsigned long long)(h->N / (g.pk[gsz] * s)) * ((s + (1u << lw) - 1) >> lw);
        const int per_sm = std::max(1, (int)(220 * 1024 / smem));
        const int grid = (int)std::min<unsigned long long>(tiles, (unsigned long long)sms * per_sm);
        rc = map_high_any(R1, grid, smem, g, j0, gsz, lw, L, j0 + gsz == n, out, cnt16);
        if (rc) return rc;
        j0 += gsz;
    }
    return 0;
}

int lns_scratch(cov_lns *h, size_t bytes)
{
    if (bytes <= h->scratch_bytes) return 0;
    if (h->scratch) cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
    if (cudaMalloc(&h->scratch, bytes) != cudaSuccess) { cudaGetLastError(); return COV_ENOMEM; }
    h->scratch_bytes = bytes;
    return 0;
}

BallGeom ball_geom(const cov_lns *h)
{
    BallGeom b;
    memset(&b, 0, sizeof b);
    b.q = h->q; b.n = h->n;
    for (int j = 0; j < h->n; j++) b.pw[j] = h->pw[j];
    b.items = h->ball; b.last = h->ball_last; b.ngroups = h->ngroups;
    return b;
}

// words in one ball of the cell
long long ball_words(const cov_lns *h)
{
    long long v = 0, c = 1;
    for (int i = 0; i <= h->R; i++) {
        v += c;
        c = c * (h->n - i) / (i + 1) * (h->q - 1);
    }
    return std::max(1LL, v);
}

// one sequence launch; st in/out through h->seq
int seq_run(cov_lns *h, SeqArgs &a, SeqState *io)
{
    a.cnt = h->cnt;
    a.b = ball_geom(h);
    a.st = h->seq;
    CK(cudaMemcpy(h->seq, io, sizeof(SeqState), cudaMemcpyHostToDevice));
    k_lns_seq<<<SEQ_CL, SEQ_NT>>>(a);
    CK(cudaGetLastError());
    CK(cudaMemcpy(io, h->seq, sizeof(SeqState), cudaMemcpyDeviceToHost));
    return 0;
}

long long count_eq(cov_lns *h, int target)
{
    if (cudaMemset(h->d_red, 0, 8) != cudaSuccess) return -1;
    k_lns_zero<<<grid_of(h->N), LNS_NT>>>(h->cnt, h->N, target, h->d_red);
    unsigned long long z = 0;
    if (cudaMemcpy(&z, h->d_red, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return (long long)z;
}

// room for a list of k words (and their flags) on the device
int list_room(cov_lns *h, int k)
{
    if (h->list) { cudaFree(h->list); h->list = nullptr; }
    if (h->flag) { cudaFree(h->flag); h->flag = nullptr; }
    CK(cudaMalloc(&h->list, (size_t)std::max(k, 1) * 4));
    CK(cudaMalloc(&h->flag, (size_t)std::max(k, 1)));
    CK(cudaMemset(h->flag, 0, (size_t)std::max(k, 1)));
    return 0;
}

// ordered extraction into device buffers (oidx, oval) of at most cap entries
int extract_dev(cov_lns *h, int32_t thr, int64_t cap, uint32_t *oidx, int32_t *oval, int64_t *found)
{
    const uint32_t chunk = 65536;
    const uint32_t nb = (h->N + chunk - 1) / chunk;
    int rc = lns_scratch(h, (size_t)nb * 8 + 16);
    if (rc) return rc;
    uint32_t *bcount = (uint32_t *)h->scratch, *boff = bcount + nb;
    k_lns_count_ge<<<nb, LNS_NT>>>(h->map, h->N, thr, chunk, bcount);
    CK(cudaGetLastError());
    std::vector<uint32_t> c(nb), o(nb);
    CK(cudaMemcpy(c.data(), bcount, (size_t)nb * 4, cudaMemcpyDeviceToHost));
    unsigned long long tot = 0;
    for (uint32_t b = 0; b < nb; b++) { o[b] = (uint32_t)std::min<unsigned long long>(tot, 0xffffffffull); tot += c[b]; }
    *found = (int64_t)tot;
    if (cap == 0 || tot == 0) return COV_OK;
    CK(cudaMemcpy(boff, o.data(), (size_t)nb * 4, cudaMemcpyHostToDevice));
    k_lns_emit_ge<<<nb, LNS_NT>>>(h->map, h->N, thr, chunk, boff, (uint32_t)cap, oidx, oval);
    CK(cudaGetLastError());
    return COV_OK;
}

}  // namespace

extern "C" {

int cov_lns_create(int32_t q, int32_t n, int32_t R, cov_lns **out)
{
    if (!out || q < 2 || q > 16 || n < 1 || n > 16 || R < 0 || R > LNS_MAXR) return COV_EINVAL;
    long long N = 1;
    for (int j = 0; j < n; j++) N *= q;
    if (N >= (1LL << 31)) return COV_ERANGE;
    if (R > n) R = n;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) { cudaGetLastError(); return COV_ENODEV; }
    cov_lns *h = new cov_lns;
    h->q = q; h->n = n; h->R = R; h->N = (uint32_t)N;
    for (int j = 0; j < n; j++) { long long p = 1; for (int k = 0; k < n - 1 - j; k++) p *= q; h->pw[j] = (uint32_t)p; }
    std::vector<uint8_t> last;
    uint32_t gcum[COV_MAXN + 2];
    std::vector<uint64_t> items = bt_items_h(q, n, R, 0, gcum, last);
    h->ngroups = gcum[std::min(R, n)];
    bool ok = cudaMalloc(&h->cnt, (size_t)N * 2) == cudaSuccess &&
              cudaMalloc(&h->map, (size_t)N * 4) == cudaSuccess &&
              cudaMalloc(&h->ball, items.size() * 8) == cudaSuccess &&
              cudaMalloc(&h->ball_last, last.size()) == cudaSuccess &&
              cudaMalloc(&h->d_red, 64 * 8) == cudaSuccess &&
              cudaMalloc(&h->cand, (size_t)CAND_CAP * 4) == cudaSuccess &&
              cudaMalloc(&h->bound, (size_t)CAND_CAP * 4) == cudaSuccess &&
              cudaMalloc(&h->fresh, (size_t)CAND_CAP * 4) == cudaSuccess &&
              cudaMalloc(&h->seq, sizeof(SeqState)) == cudaSuccess;
    for (int d = 0; ok && d <= R; d++) ok = cudaMalloc(&h->layer[d], (size_t)N * 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cov_lns_destroy(h);
        return COV_ENOMEM;
    }
    if (cudaMemcpy(h->ball, items.data(), items.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->ball_last, last.data(), last.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(h->cnt, 0, (size_t)N * 2) != cudaSuccess) {
        cov_lns_destroy(h);
        return -100;
    }
    *out = h;
    return COV_OK;
}

int cov_lns_destroy(cov_lns *h)
{
    if (!h) return COV_OK;
    cudaDeviceSynchronize();
    cudaFree(h->cnt); cudaFree(h->map); cudaFree(h->ball); cudaFree(h->ball_last); cudaFree(h->d_red);
    cudaFree(h->cand); cudaFree(h->bound); cudaFree(h->fresh); cudaFree(h->list); cudaFree(h->flag);
    cudaFree(h->seq);
    for (int d = 0; d <= LNS_MAXR; d++) cudaFree(h->layer[d]);
    cudaFree(h->scratch);
    delete h;
    return COV_OK;
}

int cov_lns_recount(cov_lns *h, const uint32_t *idx, int32_t m)
{
    if (!h || m < 0 || (m > 0 && !idx)) return COV_EINVAL;
    for (int i = 0; i < m; i++) if (idx[i] >= h->N) return COV_EINVAL;
    k_lns_zero_layer<<<grid_of(h->N), LNS_NT>>>(h->layer[0], h->N);
    CK(cudaGetLastError());
    if (m > 0) {
        int rc = lns_scratch(h, (size_t)m * 4);
        if (rc) return rc;
        CK(cudaMemcpy(h->scratch, idx, (size_t)m * 4, cudaMemcpyHostToDevice));
        k_lns_scatter<<<(m + 255) / 256, 256>>>(h->layer[0], (const uint32_t *)h->scratch, m);
        CK(cudaGetLastError());
    }
    int rc = lns_transform(h, nullptr, 0, nullptr, h->cnt);
    if (rc) return rc;
    CK(cudaDeviceSynchronize());
    return COV_OK;
}

int cov_lns_map(cov_lns *h, int32_t target)
{
    if (!h || target < 0) return COV_EINVAL;
    int rc = lns_transform(h, h->cnt, target, h->map, nullptr);
    if (rc) return rc;
    CK(cudaDeviceSynchronize());
    return COV_OK;
}

int cov_lns_map_max(cov_lns *h, int32_t *out)
{
    if (!h || !out) return COV_EINVAL;
    const int init = INT32_MIN;
    CK(cudaMemcpy(h->d_red, &init, 4, cudaMemcpyHostToDevice));
    k_lns_max<<<grid_of(h->N), LNS_NT>>>(h->map, h->N, (int *)h->d_red);
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, h->d_red, 4, cudaMemcpyDeviceToHost));
    return COV_OK;
}

int cov_lns_map_hist(cov_lns *h, int32_t nbins, int32_t vmax, int64_t *hist)
{
    if (!h || !hist || nbins < 1 || nbins > LNS_HIST_MAX || vmax < 1) return COV_EINVAL;
    int rc = lns_scratch(h, (size_t)nbins * 8);
    if (rc) return rc;
    unsigned long long *d_h = (unsigned long long *)h->scratch;
    CK(cudaMemset(d_h, 0, (size_t)nbins * 8));
    k_lns_hist<<<grid_of(h->N), LNS_NT, (size_t)nbins * 4>>>(h->map, h->N, nbins, vmax, d_h);
    CK(cudaGetLastError());
    CK(cudaMemcpy(hist, d_h, (size_t)nbins * 8, cudaMemcpyDeviceToHost));
    return COV_OK;
}

int cov_lns_map_extract(cov_lns *h, int32_t thr, int64_t cap, uint32_t *idx, int32_t *val, int64_t *found)
{
    if (!h || cap < 0 || (cap > 0 && (!idx || !val)) || !found) return COV_EINVAL;
    uint32_t *d_i = nullptr;
    int32_t *d_v = nullptr;
    if (cap > 0) {
        CK(cudaMalloc(&d_i, (size_t)cap * 4));
        if (cudaMalloc(&d_v, (size_t)cap * 4) != cudaSuccess) { cudaGetLastError(); cudaFree(d_i); return COV_ENOMEM; }
    }
    int rc = extract_dev(h, thr, cap, d_i, d_v, found);
    if (!rc && cap > 0 && *found > 0) {
        const size_t k = (size_t)std::min<int64_t>(*found, cap);
        if (cudaMemcpy(idx, d_i, k * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(val, d_v, k * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = -100;
    }
    cudaFree(d_i);
    cudaFree(d_v);
    return rc;
}

int cov_lns_map_read(cov_lns *h, const uint32_t *idx, int32_t k, int32_t *out)
{
    if (!h || k < 0 || (k > 0 && (!idx || !out))) return COV_EINVAL;
    if (k == 0) return COV_OK;
    for (int i = 0; i < k; i++) if (idx[i] >= h->N) return COV_EINVAL;
    int rc = lns_scratch(h, (size_t)k * 8);
    if (rc) return rc;
    uint32_t *d_i = (uint32_t *)h->scratch;
    int32_t *d_o = (int32_t *)(d_i + k);
    CK(cudaMemcpy(d_i, idx, (size_t)k * 4, cudaMemcpyHostToDevice));
    k_lns_read<<<(k + 255) / 256, 256>>>(h->map, d_i, k, d_o);
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, d_o, (size_t)k * 4, cudaMemcpyDeviceToHost));
    return COV_OK;
}

int cov_lns_apply(cov_lns *h, const uint32_t *idx, int32_t k, int32_t sign, int64_t *uncovered)
{
    if (!h || k < 0 || (k > 0 && !idx) || (sign != 1 && sign != -1) || !uncovered) return COV_EINVAL;
    for (int i = 0; i < k; i++) if (idx[i] >= h->N) return COV_EINVAL;
    SeqState st;
    memset(&st, 0, sizeof st);
    st.uncov = count_eq(h, 0);
    if (st.uncov < 0) return -100;
    if (k > 0) {
        int rc = list_room(h, k);
        if (rc) return rc;
        CK(cudaMemcpy(h->list, idx, (size_t)k * 4, cudaMemcpyHostToDevice));
        SeqArgs a;
        memset(&a, 0, sizeof a);
        a.mode = MODE_APPLY; a.list = h->list; a.nlist = k; a.sign = sign; a.flag = h->flag;
        a.max_steps = (long long)k + 1;
        rc = seq_run(h, a, &st);
        if (rc) return rc;
        if (st.status != SEQ_DONE) return COV_ETIMEOUT;
    }
    *uncovered = st.uncov;
    return COV_OK;
}

int cov_lns_ball(cov_lns *h, const uint32_t *idx, int32_t k, int32_t op, int32_t arg, int32_t *out)
{
    if (!h || k < 0 || (k > 0 && !idx) || op < 0 || op > 1 || (op == 0 && k > 0 && !out)) return COV_EINVAL;
    if (k == 0) return COV_OK;
    for (int i = 0; i < k; i++) if (idx[i] >= h->N) return COV_EINVAL;
    if (op == 0) {
        int rc = lns_scratch(h, (size_t)k * 8);
        if (rc) return rc;
        uint32_t *d_i = (uint32_t *)h->scratch;
        int32_t *d_o = (int32_t *)(d_i + k);
        CK(cudaMemcpy(d_i, idx, (size_t)k * 4, cudaMemcpyHostToDevice));
        k_lns_gather<<<k, LNS_NT>>>(h->cnt, d_i, k, ball_geom(h), arg, d_o);
        CK(cudaGetLastError());
        CK(cudaMemcpy(out, d_o, (size_t)k * 4, cudaMemcpyDeviceToHost));
        return COV_OK;
    }
    int64_t unc = 0;
    return cov_lns_apply(h, idx, k, arg, &unc);
}

int cov_lns_peel(cov_lns *h, const uint32_t *idx, int32_t k, uint8_t *removed, int32_t *nremoved,
                 int64_t *uncovered)
{
    if (!h || k < 0 || (k > 0 && (!idx || !removed)) || !nremoved || !uncovered) return COV_EINVAL;
    for (int i = 0; i < k; i++) if (idx[i] >= h->N) return COV_EINVAL;
    SeqState st;
    memset(&st, 0, sizeof st);
    st.uncov = count_eq(h, 0);
    if (st.uncov < 0) return -100;
    *nremoved = 0;
    if (k > 0) {
        int rc = list_room(h, k);
        if (rc) return rc;
        CK(cudaMemcpy(h->list, idx, (size_t)k * 4, cudaMemcpyHostToDevice));
        SeqArgs a;
        memset(&a, 0, sizeof a);
        a.mode = MODE_PEEL; a.list = h->list; a.nlist = k; a.flag = h->flag;
        a.max_steps = 2LL * k + 2;
        rc = seq_run(h, a, &st);
        if (rc) return rc;
        if (st.status != SEQ_DONE) return COV_ETIMEOUT;
        CK(cudaMemcpy(removed, h->flag, (size_t)k, cudaMemcpyDeviceToHost));
        *nremoved = st.removed;
    }
    *uncovered = st.uncov;
    return COV_OK;
}

// extraction threshold that keeps {map >= thr} within cap (from a histogram)
static int extract_threshold(cov_lns *h, int top, long long cap, int *thr_out)
{
    if (top <= 1) { *thr_out = 1; return 0; }
    const int nb = 1024;
    int64_t hist[1024];
    int rc = cov_lns_map_hist(h, nb, top, hist);
    if (rc) return rc;
    long long above = 0;
    int b = nb;                                      // smallest bin whose tail fits
    while (b > 0 && above + hist[b - 1] <= cap) { above += hist[b - 1]; b--; }
    // bin b holds the values v with (v-1)*nb/top == b: the first such v
    const int thr = b >= nb ? top : (int)(((long long)b * top + nb - 1) / nb) + 1;
    *thr_out = std::max(1, std::min(thr, top));
    return 0;
}

int cov_lns_greedy(cov_lns *h, int32_t room, int64_t cand_cap, uint32_t *placed, int32_t *nplaced,
                   int64_t *uncovered, int64_t *stats)
{
    if (!h || room < 0 || (room > 0 && !placed) || !nplaced || !uncovered) return COV_EINVAL;
    cand_cap = std::max<int64_t>(1, std::min<int64_t>(cand_cap > 0 ? cand_cap : CAND_CAP, CAND_CAP));
    int rc = list_room(h, room);
    if (rc) return rc;
    SeqState st;
    memset(&st, 0, sizeof st);
    st.uncov = count_eq(h, 0);
    if (st.uncov < 0) return -100;
    int total = 0;
    long long refreshes = 0, evals = 0;
    // every refresh that finds a positive gain places at least one word (the
    // first placement of a launch needs no exact count: all bounds are fresh)
    for (int guard = 0; total < room && st.uncov > 0 && guard <= 2 * room + 2; guard++) {
        // bounds: the exact gain map, extracted above a threshold that keeps
        // at most cand_cap candidates
        rc = cov_lns_map(h, 0);
        if (rc) return rc;
        refreshes++;
        int32_t top = 0;
        rc = cov_lns_map_max(h, &top);
        if (rc) return rc;
        if (top <= 0) break;
        int thr = 1;
        rc = extract_threshold(h, top, cand_cap, &thr);
        if (rc) return rc;
        int64_t found = 0;
        rc = extract_dev(h, thr, cand_cap, h->cand, h->bound, &found);
        if (rc) return rc;
        const int ncand = (int)std::min<int64_t>(found, cand_cap);
        if (ncand == 0) break;
        // every bound is exact now (epoch 1 of the launch)
        std::vector<int32_t> ones((size_t)ncand, 1);
        CK(cudaMemcpy(h->fresh, ones.data(), (size_t)ncand * 4, cudaMemcpyHostToDevice));
        SeqArgs a;
        memset(&a, 0, sizeof a);
        a.mode = MODE_GREEDY;
        a.cand = h->cand; a.bound = h->bound; a.fresh = h->fresh; a.ncand = ncand;
        // a word outside the candidates had a gain below thr at the refresh
        // (or, when even the map's maximum has more than cand_cap words, the
        // same gain and a higher position): a candidate is placed only while
        // its exact gain is at least thr, so it is always a best placement
        a.thr = thr;
        a.room = room - total;
        a.list = h->list + total;
        // a map costs about as much as N / (2 |ball|) exact counts: past
        // that many counts for one placement, refresh instead
        a.eval_cap = (int)std::max<long long>(8, std::min<long long>(4096, (long long)h->N / (2LL * ball_words(h))));
        a.max_steps = 64LL * (room - total) + 4LL * ncand + 64;
        rc = seq_run(h, a, &st);
        if (rc) return rc;
        total += st.placed;
        evals += st.evals;
        if (st.status == SEQ_GUARD) return COV_ETIMEOUT;
        if (st.status != SEQ_REFRESH) break;
    }
    if (total > 0) CK(cudaMemcpy(placed, h->list, (size_t)total * 4, cudaMemcpyDeviceToHost));
    *nplaced = total;
    *uncovered = st.uncov;
    if (stats) { stats[0] = refreshes; stats[1] = evals; }
    return COV_OK;
}

int cov_lns_uncovered(cov_lns *h, int64_t cap, uint32_t *idx, int64_t *found)
{
    if (!h || cap < 0 || (cap > 0 && !idx) || !found) return COV_EINVAL;
    // the indicator of cnt == 0 into the map, then its ordered extraction
    k_lns_indicator<<<grid_of(h->N), LNS_NT>>>(h->cnt, 0, nullptr, h->N, h->map, nullptr);
    CK(cudaGetLastError());
    std::vector<int32_t> val((size_t)std::max<int64_t>(cap, 1));
    return cov_lns_map_extract(h, 1, cap, idx, val.data(), found);
}

int cov_lns_count(cov_lns *h, int32_t target, int64_t *out)
{
    if (!h || !out || target < 0) return COV_EINVAL;
    CK(cudaMemset(h->d_red, 0, 8));
    k_lns_zero<<<grid_of(h->N), LNS_NT>>>(h->cnt, h->N, target, h->d_red);
    CK(cudaGetLastError());
    unsigned long long z = 0;
    CK(cudaMemcpy(&z, h->d_red, 8, cudaMemcpyDeviceToHost));
    *out = (int64_t)z;
    return COV_OK;
}

int cov_lns_get_cnt(cov_lns *h, uint16_t *out)
{
    if (!h || !out) return COV_EINVAL;
    CK(cudaMemcpy(out, h->cnt, (size_t)h->N * 2, cudaMemcpyDeviceToHost));
    return COV_OK;
}

int cov_lns_get_map(cov_lns *h, int32_t *out)
{
    if (!h || !out) return COV_EINVAL;
    CK(cudaMemcpy(out, h->map, (size_t)h->N * 4, cudaMemcpyDeviceToHost));
    return COV_OK;
}

}  // extern "C"
