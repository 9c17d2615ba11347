// cov_verify.cu -- GB300 (sm_103a) verification kernels for covering codes.
//
//   * exact per-word minimum distance to a code (the distance transform),
//     computed as n axis passes of the line-min recurrence
//         D'(x) = min(D(x), 1 + min_a D(x with x_j := a))
//     over uint8 values.  After the passes over axes 0..n-1, D(x) is the
//     Hamming distance from x to the nearest codeword -- the `best` array of
//     cov/verify_independent.py:144-186 -- and #{x : D(x) > R} is the
//     uncovered count that cov/verify_cov.py:109-230 returns.
//     The n passes are grouped so that HBM is swept twice, not n times:
//     the low axes of a contiguous tile, then the high axes of a column
//     strip, each group worked in shared memory.  The histogram of D is
//     folded into the last pass.
//   * coverage multiplicity cnt[x] = #{i : d(x,c_i) <= R} by marking every
//     codeword's ball (covsearch2e.c:353-380, 958-967), with 32-bit atomics
//     on packed uint16 pairs.
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include "cov_common.cuh"
#include "cov_tiles.cuh"
#include "../../include/covgpu.h"

#define DT_TILE_MAX   65536    // bytes of the contiguous low-axes tile (several CTAs per SM)
#define DT_TILE_BIG   (200 * 1024)  // a tile of one CTA per SM, used when it saves a sweep
#define DT_NT_BIG     1024     // threads of a big-tile CTA
#define DT_STRIP_MAX  98304    // bytes of a high-axes strip
#define DT_STRIP_W    32       // narrowest strip (columns); strips widen while they fit
#define DT_NT         512

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "covgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    return -(100 + (int)e_); } } while (0)

struct DtGeom {
    int q, n;
    uint32_t N;
    uint32_t pw[COV_MAXN + 1];   // pw[k] = q^k
    int inf;                     // n + 1
};

// --------------------------------------------------------- code bitmap ----
__global__ void k_dt_bitmap(const uint8_t *__restrict__ code, int M, DtGeom g, uint32_t *bm)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        uint32_t x = 0;
        for (int j = 0; j < g.n; j++) x = x * (uint32_t)g.q + code[(size_t)i * g.n + j];
        atomicOr(&bm[x >> 5], 1u << (x & 31));
    }
}

// histogram update aggregated over the lanes holding the same value
__device__ __forceinline__ void dt_hist_add(int *sh, int v)
{
    const unsigned act = __activemask();
    const unsigned same = __match_any_sync(act, v);
    if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&sh[v], __popc(same));
}

// One line-min pass over packed bytes: `nfib` fibres of Q 32-bit words, word
// a of fibre f at  base(f) + a*stride  (a < Q), base(f) = (f / inner) *
// Q*stride + (f % inner).  Each word holds 4 independent lines (one per
// byte).  The bytes are worked as two pairs of 16-bit lanes (bytes 0,2 and
// 1,3), where the minimum of three values and min(m + 1, n + 1) are single
// dynamic-programming instructions (__vimin3_u16x2, __viaddmin_u16x2).
template <int Q>
__device__ __forceinline__ void dt_pass4(uint32_t *w, int nfib, int stride, int inner, uint32_t inf4)
{
    const uint32_t inf2 = inf4 & 0x00ff00ffu;
    // f / inner by a float reciprocal: f < 2^24, so the estimate is off by
    // at most one and one correction makes it exact
    const float rinv = 1.0f / (float)inner;
    for (int f = threadIdx.x; f < nfib; f += blockDim.x) {
        int o = (int)((float)f * rinv);
        int i = f - o * inner;
        if (i < 0) { o--; i += inner; } else if (i >= inner) { o++; i -= inner; }
        uint32_t *b = w + o * Q * stride + i;
        uint32_t e[Q], d[Q];                     // bytes 0,2 and bytes 1,3 of each word
#pragma unroll
        for (int a = 0; a < Q; a++) {
            const uint32_t x = b[a * stride];
            e[a] = __byte_perm(x, 0u, 0x4240);
            d[a] = __byte_perm(x, 0u, 0x4341);
        }
        uint32_t me = e[0], md = d[0];
#pragma unroll
        for (int a = 1; a + 1 < Q; a += 2) {
            me = __vimin3_u16x2(me, e[a], e[a + 1]);
            md = __vimin3_u16x2(md, d[a], d[a + 1]);
        }
        if ((Q & 1) == 0) {
            me = __vminu2(me, e[Q - 1]);
            md = __vminu2(md, d[Q - 1]);
        }
        const uint32_t ce = __viaddmin_u16x2(me, 0x00010001u, inf2);
        const uint32_t cd = __viaddmin_u16x2(md, 0x00010001u, inf2);
#pragma unroll
        for (int a = 0; a < Q; a++)
            b[a * stride] = __byte_perm(__vminu2(e[a], ce), __vminu2(d[a], cd), 0x6240);
    }
}

// Pass 1: tiles of T = Q^k contiguous words (the low k axes), from the code
// bitmap.  In shared memory a tile is T/Q rows -- the Q words of one line of
// the lowest axis -- each padded to 4*ceil(Q/4) bytes, so that every axis
// above the lowest moves whole 32-bit words.  The lowest axis is taken while
// loading: a word is 0 on the code, 1 if its line holds a codeword, else
// n+1.  When k == n this is the whole transform and the histogram is taken
// here.
template <int Q>
__global__ void __launch_bounds__(DT_NT_BIG)
k_dt_low(DtGeom g, int k, const uint32_t *__restrict__ bm, uint8_t *__restrict__ D,
         unsigned long long *hist)
{
    extern __shared__ __align__(16) uint32_t dt_w[];
    __shared__ int sh[COV_MAXN + 2];
    constexpr int WPR = (Q + 3) >> 2;            // 32-bit words per row
    constexpr uint32_t RB = 4u * WPR;            // padded row bytes
    uint32_t T = 1;
    for (int j = 0; j < k; j++) T *= (uint32_t)Q;
    const int rows = (int)(T / (uint32_t)Q);
    const uint32_t inf = (uint32_t)g.inf, inf4 = inf * 0x01010101u;
    const uint32_t ntile = g.N / T;
    const bool last = (k == g.n) && hist != nullptr;
    uint8_t *dt_b = reinterpret_cast<uint8_t *>(dt_w);
    if (threadIdx.x < COV_MAXN + 2) sh[threadIdx.x] = 0;
    for (uint32_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const uint32_t x0 = tile * T;
        __syncthreads();
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const uint32_t xr = x0 + (uint32_t)r * (uint32_t)Q;
            // Q bits of the row from at most two bitmap words
            const uint32_t lo = __ldg(&bm[xr >> 5]);
            const uint32_t hi = ((xr & 31) + (uint32_t)Q > 32) ? __ldg(&bm[(xr >> 5) + 1]) : 0u;
            const uint32_t bits = (uint32_t)(((((uint64_t)hi << 32) | lo) >> (xr & 31)) & ((1ull << Q) - 1));
            const uint32_t fill = bits ? 1u : inf;
#pragma unroll
            for (int w = 0; w < WPR; w++) {
                uint32_t v = 0;
#pragma unroll
                for (int b = 0; b < 4; b++) {
                    const int a = 4 * w + b;
                    const uint32_t byte = a >= Q ? inf : (((bits >> a) & 1u) ? 0u : fill);
                    v |= byte << (8 * b);
                }
                dt_w[r * WPR + w] = v;
            }
        }
        __syncthreads();
        int inner = WPR;                       // rows of axis j: stride Q^(j-1) rows
        for (int j = 1; j < k; j++, inner *= Q) {
            dt_pass4<Q>(dt_w, rows / Q * WPR, inner, inner, inf4);
            __syncthreads();
        }
        // out: the tile is T contiguous bytes of D; the 4-byte-aligned
        // interior goes out as whole words (byte b of the tile is row b / Q,
        // column b % Q of the padded rows), the unaligned ends as bytes
        const uint32_t head = min((4u - (uint32_t)(reinterpret_cast<uintptr_t>(D + x0) & 3u)) & 3u, T);
        const uint32_t nw = (T - head) >> 2;
        for (uint32_t e = threadIdx.x; e < head + ((T - head) & 3u); e += blockDim.x) {
            const uint32_t b = e < head ? e : head + 4 * nw + (e - head);
            const uint32_t r = b / (uint32_t)Q;
            const uint8_t v = dt_b[r * RB + (b - r * (uint32_t)Q)];
            D[x0 + b] = v;
            if (last) dt_hist_add(sh, v);
        }
        for (uint32_t wi = threadIdx.x; wi < nw; wi += blockDim.x) {
            const uint32_t b0 = head + 4 * wi;
            uint32_t r = b0 / (uint32_t)Q, a = b0 - r * (uint32_t)Q, v = 0;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const uint32_t byte = dt_b[r * RB + a];
                v |= byte << (8 * t);
                if (last) dt_hist_add(sh, (int)byte);
                if (++a == (uint32_t)Q) { a = 0; r++; }
            }
            *reinterpret_cast<uint32_t *>(D + x0 + b0) = v;
        }
    }
    __syncthreads();
    if (last && threadIdx.x < g.n + 2 && sh[threadIdx.x])
        atomicAdd(&hist[threadIdx.x], (unsigned long long)sh[threadIdx.x]);
}

// the aligned 32-bit word that holds byte p
__device__ __forceinline__ uint32_t *dt_word_of(uint8_t *p)
{
    return reinterpret_cast<uint32_t *>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
}

// Pass 2+: the axes of group [j0, j0+gsz) (in-word strides Q^j0 .. ), for a
// strip of W = 32 << lw consecutive positions below the group: rows of W
// bytes, W/4 words, so each pass moves whole words.  W is as wide as the
// shared memory allows for the group's Q^gsz rows, so that a group of few
// rows (the last axes of a long word) still moves long contiguous runs.
// A row starts at any byte (the strides are powers of Q), so it is moved
// as 32-bit words: each loaded word is two aligned words funnel-shifted by
// the row's misalignment (the second only when it holds bytes of the row),
// and each row goes out as aligned words plus at most three bytes at either
// end.  Every word touched holds a byte of the row, so no access leaves it.
template <int Q>
__global__ void __launch_bounds__(DT_NT)
k_dt_high(DtGeom g, int j0, int gsz, int lw, int last_, uint8_t *__restrict__ D, unsigned long long *hist)
{
    const bool last = last_ && hist != nullptr;
    extern __shared__ __align__(16) uint32_t dt_w[];
    __shared__ int sh[COV_MAXN + 2];
    const int lwb = lw + 5;                      // log2 of the strip width in bytes
    const int lww = lwb - 2;                     // log2 of the words per row
    const uint32_t W = 1u << lwb;
    const uint32_t WW = W >> 2;
    uint8_t *dt_b = reinterpret_cast<uint8_t *>(dt_w);
    const uint32_t inf4 = (uint32_t)g.inf * 0x01010101u;
    uint32_t s = 1;                              // stride of the lowest axis in the group
    for (int j = 0; j < j0; j++) s *= (uint32_t)Q;
    uint32_t rows = 1;
    for (int j = 0; j < gsz; j++) rows *= (uint32_t)Q;
    const uint32_t span = rows * s;              // words spanned by one value of the outer digits
    const uint32_t outer = g.N / span;
    const uint32_t nstrip = (s + W - 1) >> lwb;
    const unsigned long long ntiles = (unsigned long long)outer * nstrip;
    if (threadIdx.x < COV_MAXN + 2) sh[threadIdx.x] = 0;
    const uint32_t totw = rows << lww;
    for (unsigned long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t o = (uint32_t)(tile / nstrip);
        const uint32_t c0 = (uint32_t)(tile - (unsigned long long)o * nstrip) << lwb;
        const uint32_t w = min(W, s - c0);       // bytes of each row in this strip
        uint8_t *const Db = D + (size_t)o * span + c0;
        __syncthreads();
        // word k of row r: bytes 4k..4k+3 of the row at Db + r*s (n+1
        // past w); eight words of a thread in flight before their stores
        for (uint32_t e0 = threadIdx.x; e0 < totw; e0 += 8 * blockDim.x) {
            uint32_t v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const uint32_t e = e0 + (uint32_t)u * blockDim.x;
                const uint32_t r = e >> lww, c = (e & (WW - 1)) << 2;
                v[u] = inf4;
                if (e < totw && c < w) {
                    uint8_t *p = Db + (size_t)r * s + c;
                    const uint32_t m = (uint32_t)(reinterpret_cast<uintptr_t>(p) & 3u);
                    const uint32_t need = min(4u, w - c);
                    const uint32_t *pa = dt_word_of(p);
                    const uint32_t lo = pa[0];
                    const uint32_t hi = m + need > 4u ? pa[1] : 0u;
                    uint32_t x = __funnelshift_r(lo, hi, 8u * m);
                    if (need < 4u) {
                        const uint32_t keep = (1u << (8u * need)) - 1u;
                        x = (x & keep) | (inf4 & ~keep);
                    }
                    v[u] = x;
                }
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const uint32_t e = e0 + (uint32_t)u * blockDim.x;
                if (e < totw) dt_w[e] = v[u];
            }
        }
        __syncthreads();
        int inner = (int)WW;                     // row stride Q^j
        for (int j = 0; j < gsz; j++, inner *= Q) {
            dt_pass4<Q>(dt_w, (int)(rows / (uint32_t)Q) * (int)WW, inner, inner, inf4);
            __syncthreads();
        }
        // out: row r's aligned words from its first 4-byte boundary on, then
        // the ends (at most 3 bytes each) by the thread of the row's last word
        for (uint32_t e = threadIdx.x; e < totw; e += blockDim.x) {
            const uint32_t r = e >> lww, k = e & (WW - 1);
            uint8_t *p0 = Db + (size_t)r * s;
            const uint32_t head = min((4u - (uint32_t)(reinterpret_cast<uintptr_t>(p0) & 3u)) & 3u, w);
            const uint32_t nwr = (w - head) >> 2;
            if (k < nwr) {
                const uint32_t lo = dt_w[(r << lww) + k];
                const uint32_t hi = head ? dt_w[(r << lww) + k + 1] : 0u;
                const uint32_t x = __funnelshift_r(lo, hi, 8u * head);
                *reinterpret_cast<uint32_t *>(p0 + head + 4 * k) = x;
                if (last) {
#pragma unroll
                    for (int b = 0; b < 4; b++) dt_hist_add(sh, (int)((x >> (8 * b)) & 0xffu));
                }
            }
            if (k == WW - 1) {
                const uint8_t *row = dt_b + ((size_t)r << lwb);
                for (uint32_t b = 0; b < head; b++) {
                    p0[b] = row[b];
                    if (last) atomicAdd(&sh[row[b]], 1);
                }
                for (uint32_t b = head + 4 * nwr; b < w; b++) {
                    p0[b] = row[b];
                    if (last) atomicAdd(&sh[row[b]], 1);
                }
            }
        }
    }
    __syncthreads();
    if (last && threadIdx.x < g.n + 2 && sh[threadIdx.x])
        atomicAdd(&hist[threadIdx.x], (unsigned long long)sh[threadIdx.x]);
}

// the transform kernels of every q, for a runtime q
template <template <int> class F, class... A>
int dt_for_q(int q, A... a)
{
    switch (q) {
    case 2: return F<2>::run(a...);   case 3: return F<3>::run(a...);   case 4: return F<4>::run(a...);
    case 5: return F<5>::run(a...);   case 6: return F<6>::run(a...);   case 7: return F<7>::run(a...);
    case 8: return F<8>::run(a...);   case 9: return F<9>::run(a...);   case 10: return F<10>::run(a...);
    case 11: return F<11>::run(a...); case 12: return F<12>::run(a...); case 13: return F<13>::run(a...);
    case 14: return F<14>::run(a...); case 15: return F<15>::run(a...); case 16: return F<16>::run(a...);
    default: return COV_EINVAL;
    }
}

template <int Q> struct DtAttrs {
    static int run()
    {
        if (cudaFuncSetAttribute(k_dt_low<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, DT_TILE_BIG) != cudaSuccess ||
            cudaFuncSetAttribute(k_dt_high<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, DT_STRIP_MAX) != cudaSuccess)
            return -(100 + (int)cudaGetLastError());
        return 0;
    }
};
template <int Q> struct DtLow {
    static int run(int grid, int nt, size_t smem, cudaStream_t st, DtGeom g, int k, const uint32_t *bm,
                   uint8_t *D, unsigned long long *hist)
    {
        k_dt_low<Q><<<grid, nt, smem, st>>>(g, k, bm, D, hist);
        return 0;
    }
};
template <int Q> struct DtHigh {
    static int run(int grid, size_t smem, cudaStream_t st, DtGeom g, int j0, int gsz, int lw, int last,
                   uint8_t *D, unsigned long long *hist)
    {
        k_dt_high<Q><<<grid, DT_NT, smem, st>>>(g, j0, gsz, lw, last, D, hist);
        return 0;
    }
};

__global__ void k_count_above(const uint8_t *__restrict__ D, uint32_t N, int R, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        c += D[x] > R;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ------------------------------------------------ coverage multiplicity ----
__global__ void k_pack_code(const uint8_t *__restrict__ code, int M, int n, uint64_t *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        uint64_t v = 0;
        for (int j = 0; j < n; j++) v |= (uint64_t)code[(size_t)i * n + j] << (4 * j);
        out[i] = v;
    }
}

struct CountGeom {
    int q, n, R, M, nh, nl;
    uint32_t tw;                       // q^nl words per tile
    uint32_t nitems;                   // ball groups (their last positions follow them)
    uint32_t pw[COV_MAXN];             // q^(n-1-j)
    uint32_t vcum[COV_MAXN + 2];
};

// cnt[x] = #{i : d(x, c_i) <= R} saturated at 65535 (the cnt[] of
// covsearch2e.c:958-967, the OUT=2 map of cov/gemm2/dct.cu:360-411), one CTA
// per tile (cov_tiles.cuh); the tile's uncovered words are counted too.
template <int Q>
__global__ void __launch_bounds__(BT_NT) k_count_tiles(CountGeom g, const uint64_t *__restrict__ code,
                                                       const uint64_t *__restrict__ items, uint16_t *cnt,
                                                       unsigned long long *zeros)
{
    extern __shared__ __align__(16) unsigned char ct_raw[];
    uint64_t *lpc = (uint64_t *)ct_raw;
    uint32_t *lid = (uint32_t *)(lpc + BT_LCH);
    uint32_t *lbase = lid + BT_LCH;
    uint32_t *tile = lbase + BT_LCH;
    __shared__ int gcnt[COV_MAXN + 2], gpos[COV_MAXN + 2], gfill[COV_MAXN + 2];
    uint64_t hp = 0;
    {
        uint32_t t = blockIdx.x;
        for (int j = g.nh - 1; j >= 0; --j) { hp |= (uint64_t)(t % (uint32_t)g.q) << (4 * j); t /= (uint32_t)g.q; }
    }
    for (uint32_t x = threadIdx.x; x < g.tw; x += BT_NT) tile[x] = 0;
    BtScratch sc{lpc, lid, lbase, gcnt, gpos, gfill};
    bt_mark_tile<Q>(tile, g.q, g.n, g.R, g.M, code, g.pw, g.nh, g.nl, items,
                 reinterpret_cast<const uint8_t *>(items + g.nitems), g.vcum, hp, sc,
                 [](uint32_t) { return 1u; });
    unsigned long long z = 0;
    uint16_t *out = cnt + (size_t)blockIdx.x * g.tw;
    for (uint32_t x = threadIdx.x; x < g.tw; x += BT_NT) {
        const uint32_t v = tile[x];
        out[x] = (uint16_t)min(v, 65535u);
        z += v == 0;
    }
    for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
    if ((threadIdx.x & 31) == 0 && z && zeros) atomicAdd(zeros, z);
}

// ------------------------------------------------------------ finisher ----
struct FinishGeom {
    int q, n, R, M;
    uint32_t N;
    uint32_t pw[COV_MAXN];             // q^(n-1-j)
    uint32_t ngroups;                  // ball groups of radius <= R (cov_tiles.cuh, nh = 0)
};

__device__ __forceinline__ uint64_t fin_xorshift(uint64_t r)
{
    r ^= r << 13;
    r ^= r >> 7;
    r ^= r << 17;
    return r;
}

// +1 (saturating) over the ball of the packed word pc into cnt; all threads
__device__ void fin_mark(const FinishGeom &g, uint16_t *cnt, uint64_t pc, const uint64_t *items,
                         const uint8_t *last)
{
    uint32_t base = 0;
    for (int j = 0; j < g.n; j++) base += (uint32_t)cov_nib(pc, j) * g.pw[j];
    for (uint32_t it = threadIdx.x; it < g.ngroups; it += blockDim.x) {
        uint64_t sp = items[it];
        int off = (int)base;
        while (sp) {
            const int j = (__ffsll((long long)sp) - 1) >> 2;
            const int dig = (int)((sp >> (4 * j)) & 15u) - 1;
            sp &= ~(15ull << (4 * j));
            const int cj = cov_nib(pc, j);
            off += (dig + (dig >= cj) - cj) * (int)g.pw[j];
        }
        const int lj = last[it];
        if (lj == 0xff) {
            if (cnt[off] != 0xffffu) cnt[off]++;
        } else {
            const int step = (int)g.pw[lj], cj = cov_nib(pc, lj);
            int o2 = off - cj * step;
            for (int v = 0; v < g.q; v++, o2 += step)
                if (v != cj && cnt[o2] != 0xffffu) cnt[o2]++;
        }
    }
}

// Top-up of covcount (cov/engine/covcount.c:163-195), one CTA: words m0..M-1
// of code[] (packed) are chosen in order -- the first of 64 xorshift64
// draws (seeded 88172645463325252 ^ m0) that is still uncovered, else the
// first uncovered word from the scan position on, else any draw not yet in
// the code -- and each one's ball is marked before the next is chosen.
// Words of one ball are distinct, so the marking needs no atomics.
__global__ void __launch_bounds__(512) k_topup(FinishGeom g, uint16_t *cnt, uint64_t *code, int m0,
                                               const uint64_t *__restrict__ items,
                                               const uint8_t *__restrict__ last)
{
    __shared__ uint64_t draw_st[64];
    __shared__ uint32_t draw_x[64];
    __shared__ unsigned hit[2];
    __shared__ uint64_t s_rs;
    __shared__ long long s_w, s_scan;
    __shared__ int s_dup;
    __shared__ uint64_t s_new;
    if (threadIdx.x == 0) { s_rs = 88172645463325252ull ^ (uint64_t)m0; s_scan = 0; }
    __syncthreads();
    for (int m = m0; m < g.M; m++) {
        if (threadIdx.x == 0) {
            uint64_t r = s_rs;
            for (int t = 0; t < 64; t++) { r = fin_xorshift(r); draw_st[t] = r; draw_x[t] = (uint32_t)(r % g.N); }
        }
        __syncthreads();
        if (threadIdx.x < 64) {
            const unsigned b = __ballot_sync(0xffffffffu, cnt[draw_x[threadIdx.x]] == 0);
            if ((threadIdx.x & 31) == 0) hit[threadIdx.x >> 5] = b;
        }
        __syncthreads();
        int f = -1;
        if (hit[0]) f = __ffs(hit[0]) - 1;
        else if (hit[1]) f = 32 + __ffs(hit[1]) - 1;
        long long w = -1;
        if (f >= 0) {
            w = draw_x[f];
        } else {
            // first zero at or after the scan position, in chunks of the block
            for (long long x0 = s_scan; x0 < (long long)g.N && w < 0; x0 += blockDim.x) {
                const long long x = x0 + threadIdx.x;
                const int z = x < (long long)g.N && cnt[x] == 0;
                const int any = __syncthreads_or(z);
                if (any) {
                    if (threadIdx.x == 0) s_w = 0x7fffffffffffffffll;
                    __syncthreads();
                    if (z) atomicMin((unsigned long long *)&s_w, (unsigned long long)x);
                    __syncthreads();
                    w = s_w;
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_rs = f >= 0 ? draw_st[f] : draw_st[63];
            s_scan = f >= 0 ? s_scan : (w >= 0 ? w : (long long)g.N);
        }
        __syncthreads();
        if (w >= 0) {
            if (threadIdx.x == 0) {
                uint64_t pk = 0;
                uint32_t y = (uint32_t)w;
                for (int j = g.n - 1; j >= 0; j--) { pk |= (uint64_t)(y % (uint32_t)g.q) << (4 * j); y /= (uint32_t)g.q; }
                s_new = pk;
            }
        } else {
            // everything covered: any draw that is not yet a codeword
            for (;;) {
                if (threadIdx.x == 0) {
                    s_rs = fin_xorshift(s_rs);
                    uint32_t y = (uint32_t)(s_rs % g.N);
                    uint64_t pk = 0;
                    for (int j = g.n - 1; j >= 0; j--) { pk |= (uint64_t)(y % (uint32_t)g.q) << (4 * j); y /= (uint32_t)g.q; }
                    s_new = pk;
                    s_dup = 0;
                }
                __syncthreads();
                for (int i = threadIdx.x; i < m; i += blockDim.x)
                    if (code[i] == s_new) s_dup = 1;
                __syncthreads();
                if (!s_dup) break;
                __syncthreads();
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) code[m] = s_new;
        fin_mark(g, cnt, s_new, items, last);
        __syncthreads();
    }
}

__global__ void k_count_zero16(const uint16_t *cnt, uint32_t N, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        c += cnt[x] == 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ============================================================ host ========
namespace {

long long ipw(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }

int geom(int q, int n, DtGeom &g)
{
    if (q < 2 || q > 16 || n < 1 || n > 16) return COV_EINVAL;
    long long N = ipw(q, n);
    if (N >= (1LL << 32) - 1) return COV_EINVAL;
    g.q = q; g.n = n; g.N = (uint32_t)N; g.inf = n + 1;
    for (int k = 0; k <= COV_MAXN; k++) g.pw[k] = (uint32_t)std::min<long long>(ipw(q, k), 0xffffffffLL);
    return 0;
}

CovDeviceFlags g_dt_attr;   // shared-memory opt-in of the transform kernels, per device
CovDeviceFlags g_ct_attr;   // the same for the tile count

// the tile count of the alphabet size q (a kernel of its own for q = 5..8)
void ct_launch(int q, unsigned grid, size_t smem, cudaStream_t st, const CountGeom &g, const uint64_t *code,
               const uint64_t *items, uint16_t *cnt)
{
    switch (q) {
#define CT_LAUNCH_Q(QQ) case QQ: k_count_tiles<QQ><<<grid, BT_NT, smem, st>>>(g, code, items, cnt, nullptr); break;
    BT_Q_LIST(CT_LAUNCH_Q)
#undef CT_LAUNCH_Q
    default: k_count_tiles<0><<<grid, BT_NT, smem, st>>>(g, code, items, cnt, nullptr); break;
    }
}

int ct_attrs()
{
    int dev = 0;
    if (g_ct_attr.done(dev)) return 0;
    CK(cudaFuncSetAttribute(k_count_tiles<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)bt_smem_bytes(BT_MAX)));
#define CT_ATTR_Q(QQ) \
    CK(cudaFuncSetAttribute(k_count_tiles<QQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt_smem_bytes(BT_MAX)));
    BT_Q_LIST(CT_ATTR_Q)
#undef CT_ATTR_Q
    g_ct_attr.set(dev);
    return 0;
}

// the transform on device buffers; hist (device, n+2 entries) may be null
int dt_run(const DtGeom &g, const uint8_t *d_code, int M, uint8_t *d_D, unsigned long long *d_hist,
           uint32_t *d_bm, cudaStream_t st)
{
    int dev = 0;
    if (!g_dt_attr.done(dev)) {
        for (int q = 2; q <= COV_MAXQ; q++) {
            const int rc = dt_for_q<DtAttrs>(q);
            if (rc) return rc;
        }
        g_dt_attr.set(dev);
    }
    CK(cudaMemsetAsync(d_bm, 0, (size_t)((g.N + 31) / 32) * 4, st));
    if (M > 0) {
        k_dt_bitmap<<<std::min(1024, (M + 255) / 256), 256, 0, st>>>(d_code, M, g, d_bm);
        CK(cudaGetLastError());
    }
    // low group: as many axes as fit a tile
    const long long q4 = (g.q + 3) / 4 * 4;      // padded bytes of one lowest-axis line
    auto low_bytes = [&](int kk) { return (long long)g.pw[kk] / g.q * q4; };
    // HBM sweeps of the strip passes after a low tile of kk axes
    auto strip_sweeps = [&](int kk) {
        int sw = 0, j = kk;
        while (j < g.n) {
            int gz = 0;
            while (j + gz < g.n && (long long)g.pw[gz + 1] * DT_STRIP_W <= DT_STRIP_MAX) gz++;
            j += std::max(gz, 1);
            sw++;
        }
        return sw;
    };
    int k = 1;
    while (k < g.n && low_bytes(k + 1) <= DT_TILE_MAX) k++;
    // a bigger tile (one CTA per SM, twice the threads) only where it saves a sweep
    int kb = k;
    while (kb < g.n && low_bytes(kb + 1) <= DT_TILE_BIG) kb++;
    const bool big = strip_sweeps(kb) < strip_sweeps(k);
    if (big) k = kb;
    const int sms = std::max(1, cov_sm_count());
    const uint32_t ntile = g.N / g.pw[k];
    {
        int grid = (int)std::min<uint32_t>(ntile, (uint32_t)sms * (big ? 1 : 4));
        dt_for_q<DtLow>(g.q, grid, big ? DT_NT_BIG : DT_NT, (size_t)low_bytes(k), st, g, k,
                        (const uint32_t *)d_bm, d_D, d_hist);
        CK(cudaGetLastError());
    }
    // high groups
    int j0 = k;
    while (j0 < g.n) {
        int gsz = 0;
        while (j0 + gsz < g.n && (long long)g.pw[gsz + 1] * DT_STRIP_W <= DT_STRIP_MAX) gsz++;
        if (gsz == 0) return COV_EINVAL;
        int last = (j0 + gsz == g.n);
        const uint32_t s = g.pw[j0];
        // widest power-of-two strip (>= DT_STRIP_W bytes) the shared memory
        // holds for these rows, but no wider than the group's stride needs
        int lw = 0;
        while ((long long)g.pw[gsz] * (DT_STRIP_W << (lw + 1)) <= DT_STRIP_MAX &&
               (uint32_t)(DT_STRIP_W << lw) < s)
            lw++;
        const uint32_t W = (uint32_t)DT_STRIP_W << lw;
        const unsigned long long tiles = (unsigned long long)(g.N / (g.pw[gsz] * s)) * ((s + W - 1) / W);
        int grid = (int)std::min<unsigned long long>(tiles, (unsigned long long)sms * 4);
        dt_for_q<DtHigh>(g.q, grid, (size_t)g.pw[gsz] * W, st, g, j0, gsz, lw, last, d_D, d_hist);
        CK(cudaGetLastError());
        j0 += gsz;
    }
    return 0;
}

}  // namespace

extern "C" {

int cov_mindist_dev(int32_t q, int32_t n, const uint8_t *d_code, int32_t M, uint8_t *d_dist, void *stream)
{
    DtGeom g;
    int rc = geom(q, n, g);
    if (rc) return rc;
    if (M < 0 || (M > 0 && !d_code) || !d_dist) return COV_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t *bm = nullptr;
    CK(cudaMallocAsync(&bm, (size_t)((g.N + 31) / 32) * 4, st));
    rc = dt_run(g, d_code, M, d_dist, nullptr, bm, st);
    cudaFreeAsync(bm, st);
    return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free distance transform.
//
// For callers that must not allocate device memory themselves: a host runtime
// whose device memory is entirely owned by another allocator (for example a
// framework's caching allocator that has reserved the whole GPU), or code
// that runs where an allocation would break the surrounding contract (inside
// an out-of-memory handler).  The one scratch buffer the transform needs --
// the bitmap of codeword positions -- lives in a file-scope device array
// instead of being allocated per call.
//
//  * Limit: q^n <= COV_DT_STATIC_MAX_WORDS (2^26 words, an 8 MiB bitmap that
//    every GPU which loads the library keeps until the process exits).
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it.
//  * Every call uses the same array and clears it before use: two calls
//    whose work overlaps on the GPU (different streams, no ordering) race.
#define COV_DT_STATIC_MAX_WORDS (1u << 26)
#define COV_DT_STATIC_MAX_DEVICES 64

static __device__ __align__(256) uint32_t g_dt_static_bitmap[COV_DT_STATIC_MAX_WORDS / 32];
static uint32_t *g_dt_static_addr[COV_DT_STATIC_MAX_DEVICES];   // per device, host side

int cov_mindist_dev_static(int32_t q, int32_t n, const uint8_t *d_code, int32_t M, uint8_t *d_dist, void *stream)
{
    DtGeom g;
    int rc = geom(q, n, g);
    if (rc) return rc;
    if (g.N > COV_DT_STATIC_MAX_WORDS) {
        fprintf(stderr, "cov_mindist_dev_static: q^n = %u words exceeds the %u-word limit of the static scratch\n",
                g.N, COV_DT_STATIC_MAX_WORDS);
        return COV_ERANGE;
    }
    if (M < 0 || (M > 0 && !d_code) || !d_dist) return COV_EINVAL;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= COV_DT_STATIC_MAX_DEVICES) return COV_ENODEV;
    if (!g_dt_static_addr[dev]) {
        // the array's name is only a host-side stand-in: ask the runtime for
        // its address on the current device
        void *ptr = nullptr;
        CK(cudaGetSymbolAddress(&ptr, g_dt_static_bitmap));
        g_dt_static_addr[dev] = (uint32_t *)ptr;
    }
    return dt_run(g, d_code, M, d_dist, nullptr, g_dt_static_addr[dev], (cudaStream_t)stream);
}

int64_t cov_count_above_dev(int32_t q, int32_t n, const uint8_t *d_dist, int32_t R, void *stream)
{
    DtGeom g;
    int rc = geom(q, n, g);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long *d_c = nullptr, h = 0;
    CK(cudaMallocAsync(&d_c, 8, st));
    CK(cudaMemsetAsync(d_c, 0, 8, st));
    k_count_above<<<std::max(1, cov_sm_count()) * 8, 256, 0, st>>>(d_dist, g.N, R, d_c);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&h, d_c, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaFreeAsync(d_c, st));
    CK(cudaStreamSynchronize(st));
    return (int64_t)h;
}

int cov_mindist(int32_t q, int32_t n, const uint8_t *code, int32_t M, uint8_t *dist, int64_t *hist,
                int32_t *radius)
{
    DtGeom g;
    int rc = geom(q, n, g);
    if (rc) return rc;
    if (M < 0 || (M > 0 && !code)) return COV_EINVAL;
    for (long long i = 0; i < (long long)M * n; i++) if (code[i] >= q) return COV_EINVAL;
    cudaStream_t st = nullptr;
    uint8_t *d_code = nullptr, *d_D = nullptr;
    uint32_t *d_bm = nullptr;
    unsigned long long *d_h = nullptr;
    const size_t cb = (size_t)std::max(M, 1) * n;
    if (cudaMalloc(&d_code, cb) != cudaSuccess || cudaMalloc(&d_D, g.N) != cudaSuccess ||
        cudaMalloc(&d_bm, (size_t)((g.N + 31) / 32) * 4) != cudaSuccess ||
        cudaMalloc(&d_h, 8 * (COV_MAXN + 2)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_code); cudaFree(d_D); cudaFree(d_bm); cudaFree(d_h);
        return COV_ENOMEM;
    }
    auto done = [&](int r) { cudaFree(d_code); cudaFree(d_D); cudaFree(d_bm); cudaFree(d_h); return r; };
    if (M > 0 && cudaMemcpy(d_code, code, (size_t)M * n, cudaMemcpyHostToDevice) != cudaSuccess) return done(-100);
    if (cudaMemset(d_h, 0, 8 * (COV_MAXN + 2)) != cudaSuccess) return done(-100);
    rc = dt_run(g, d_code, M, d_D, d_h, d_bm, st);
    if (rc) return done(rc);
    unsigned long long hh[COV_MAXN + 2];
    cudaError_t e = cudaMemcpy(hh, d_h, 8 * (COV_MAXN + 2), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return done(-(100 + (int)e));
    if (dist) {
        e = cudaMemcpy(dist, d_D, g.N, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return done(-(100 + (int)e));
    }
    int rad = 0;
    for (int v = 0; v <= n + 1; v++) {
        if (hist) hist[v] = (int64_t)hh[v];
        if (hh[v]) rad = v;
    }
    if (radius) *radius = rad;
    return done(COV_OK);
}

int cov_verify(int32_t q, int32_t n, int32_t R, const uint8_t *code, int32_t M, int64_t *uncovered)
{
    if (R < 0) return COV_EINVAL;
    int64_t hist[COV_MAXN + 2];
    int rc = cov_mindist(q, n, code, M, nullptr, hist, nullptr);
    if (rc) return rc;
    int64_t u = 0;
    for (int v = R + 1; v <= n + 1; v++) u += hist[v];
    if (uncovered) *uncovered = u;
    return COV_OK;
}

int cov_count_dev(int32_t q, int32_t n, int32_t R, const uint8_t *d_code, int32_t M, uint16_t *d_cnt,
                  void *stream)
{
    DtGeom dg;
    int rc = geom(q, n, dg);
    if (rc) return rc;
    if (R < 0 || M < 0 || M > 65535 || (M > 0 && !d_code) || !d_cnt) return COV_EINVAL;
    if (R > n) R = n;
    cudaStream_t st = (cudaStream_t)stream;
    rc = ct_attrs();
    if (rc) return rc;
    CountGeom g;
    memset(&g, 0, sizeof g);
    g.q = q; g.n = n; g.R = R; g.M = M;
    bt_geom(q, n, &g.nh, &g.nl);
    g.tw = (uint32_t)ipw(q, g.nl);
    for (int j = 0; j < n; j++) g.pw[j] = dg.pw[n - 1 - j];
    std::vector<uint8_t> last;
    std::vector<uint64_t> items = bt_items_h(q, n, R, g.nh, g.vcum, last);
    g.nitems = (uint32_t)items.size();
    // one scratch allocation: the ball groups, their last positions, then
    // the packed code
    void *tmp = nullptr;
    const size_t ib = items.size() * 8, lb = (last.size() + 7) / 8 * 8;
    CK(cudaMallocAsync(&tmp, ib + lb + (size_t)std::max(M, 1) * 8, st));
    uint64_t *d_items = (uint64_t *)tmp, *d_pk = d_items + (ib + lb) / 8;
    CK(cudaMemcpyAsync(d_items, items.data(), ib, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_items + items.size(), last.data(), last.size(), cudaMemcpyHostToDevice, st));
    if (M > 0) {
        k_pack_code<<<std::min(1024, (M + 255) / 256), 256, 0, st>>>(d_code, M, n, d_pk);
        CK(cudaGetLastError());
    }
    ct_launch(q, (unsigned)ipw(q, g.nh), bt_smem_bytes(g.tw), st, g, d_pk, d_items, d_cnt);
    CK(cudaGetLastError());
    // items is pageable host memory: wait before it goes out of scope
    CK(cudaStreamSynchronize(st));
    CK(cudaFreeAsync(tmp, st));
    return COV_OK;
}

// The finisher of cov/engine/covcount.c: de-duplicate the m words (first
// occurrences kept), top them up to M distinct words and count the
// uncovered words of the result.  fast: top-up in base-q counting order, no
// coverage (uncovered = -1).
int cov_finish(int32_t q, int32_t n, int32_t R, int32_t M, const uint8_t *code, int32_t m, int32_t fast,
               uint8_t *out, int32_t *words, int64_t *uncovered)
{
    DtGeom dg;
    int rc = geom(q, n, dg);
    if (rc) return rc;
    if (R < 0 || M < 1 || m < 0 || (m > 0 && !code) || !out) return COV_EINVAL;
    if ((long long)M > (long long)dg.N) return COV_EINVAL;           // no M distinct words exist
    if (R > n) R = n;
    for (long long i = 0; i < (long long)m * n; i++) if (code[i] >= q) return COV_EINVAL;
    std::vector<uint64_t> pk;
    {
        pk.reserve((size_t)std::min(m, M));
        // covcount reads at most M words, then drops the repeats among them
        for (int i = 0; i < std::min(m, M); i++) {
            uint64_t v = 0;
            for (int j = 0; j < n; j++) v |= (uint64_t)code[(size_t)i * n + j] << (4 * j);
            if (std::find(pk.begin(), pk.end(), v) == pk.end()) pk.push_back(v);
        }
    }
    const int m0 = (int)pk.size();
    auto unpack = [&](const std::vector<uint64_t> &v) {
        for (int i = 0; i < M; i++)
            for (int j = 0; j < n; j++) out[(size_t)i * n + j] = (uint8_t)((v[i] >> (4 * j)) & 15u);
    };
    if (fast) {
        // base-q counting order, skipping words already present
        std::vector<uint64_t> v = pk;
        for (uint32_t x = 0; (int)v.size() < M; x++) {
            uint64_t w = 0;
            uint32_t y = x;
            for (int j = n - 1; j >= 0; j--) { w |= (uint64_t)(y % (uint32_t)q) << (4 * j); y /= (uint32_t)q; }
            if (std::find(v.begin(), v.end(), w) == v.end()) v.push_back(w);
        }
        unpack(v);
        if (words) *words = M;
        if (uncovered) *uncovered = -1;
        return COV_OK;
    }
    if (dg.N > 1200000000u) return COV_ERANGE;                        // covcount's limit without --fast
    rc = ct_attrs();
    if (rc) return rc;
    // tile count of the deduplicated words
    CountGeom g;
    memset(&g, 0, sizeof g);
    g.q = q; g.n = n; g.R = R; g.M = m0;
    bt_geom(q, n, &g.nh, &g.nl);
    g.tw = (uint32_t)ipw(q, g.nl);
    for (int j = 0; j < n; j++) g.pw[j] = dg.pw[n - 1 - j];
    std::vector<uint8_t> tlast, blast;
    std::vector<uint64_t> titems = bt_items_h(q, n, R, g.nh, g.vcum, tlast);
    g.nitems = (uint32_t)titems.size();
    // whole-ball groups for the top-up (no high digits)
    uint32_t bcum[COV_MAXN + 2];
    std::vector<uint64_t> bitems = bt_items_h(q, n, R, 0, bcum, blast);
    FinishGeom fg;
    memset(&fg, 0, sizeof fg);
    fg.q = q; fg.n = n; fg.R = R; fg.M = M; fg.N = dg.N;
    for (int j = 0; j < n; j++) fg.pw[j] = dg.pw[n - 1 - j];
    fg.ngroups = bcum[std::min(R, n)];
    const size_t tib = titems.size() * 8, tlb = (tlast.size() + 7) / 8 * 8;
    const size_t bib = bitems.size() * 8, blb = (blast.size() + 7) / 8 * 8;
    const size_t cb = ((size_t)dg.N * 2 + 15) / 16 * 16;
    char *buf = nullptr;
    if (cudaMalloc(&buf, tib + tlb + bib + blb + (size_t)M * 8 + cb + 16) != cudaSuccess) {
        cudaGetLastError();
        return COV_ENOMEM;
    }
    uint64_t *d_ti = (uint64_t *)buf;
    uint64_t *d_bi = (uint64_t *)(buf + tib + tlb);
    uint8_t *d_bl = (uint8_t *)(buf + tib + tlb + bib);
    uint64_t *d_code = (uint64_t *)(buf + tib + tlb + bib + blb);
    uint16_t *d_cnt = (uint16_t *)(buf + tib + tlb + bib + blb + (size_t)M * 8);
    unsigned long long *d_z = (unsigned long long *)(buf + tib + tlb + bib + blb + (size_t)M * 8 + cb);
    auto done = [&](int r) { cudaFree(buf); return r; };
    cudaError_t e = cudaSuccess;
    e = cudaMemcpy(d_ti, titems.data(), tib, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_ti + titems.size(), tlast.data(), tlast.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_bi, bitems.data(), bib, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_bl, blast.data(), blast.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && m0 > 0) e = cudaMemcpy(d_code, pk.data(), (size_t)m0 * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_z, 0, 8);
    if (e != cudaSuccess) return done(-(100 + (int)e));
    ct_launch(q, (unsigned)ipw(q, g.nh), bt_smem_bytes(g.tw), 0, g, d_code, d_ti, d_cnt);
    e = cudaGetLastError();
    if (e == cudaSuccess && m0 < M) {
        k_topup<<<1, 512>>>(fg, d_cnt, d_code, m0, d_bi, d_bl);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_count_zero16<<<std::max(1, cov_sm_count()) * 4, 256>>>(d_cnt, dg.N, d_z);
        e = cudaGetLastError();
    }
    std::vector<uint64_t> v((size_t)M);
    unsigned long long z = 0;
    if (e == cudaSuccess) e = cudaMemcpy(v.data(), d_code, (size_t)M * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&z, d_z, 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return done(-(100 + (int)e));
    unpack(v);
    if (words) *words = M;
    if (uncovered) *uncovered = (int64_t)z;
    return done(COV_OK);
}

int cov_count(int32_t q, int32_t n, int32_t R, const uint8_t *code, int32_t M, uint16_t *cnt,
              int64_t *uncovered)
{
    DtGeom g;
    int rc = geom(q, n, g);
    if (rc) return rc;
    if (R < 0 || M < 0 || M > 65535 || (M > 0 && !code)) return COV_EINVAL;
    for (long long i = 0; i < (long long)M * n; i++) if (code[i] >= q) return COV_EINVAL;
    uint8_t *d_code = nullptr;
    uint16_t *d_cnt = nullptr;
    const size_t nb = ((size_t)g.N + 1) / 2 * 4;     // whole 32-bit pairs
    if (cudaMalloc(&d_code, (size_t)std::max(M, 1) * n) != cudaSuccess ||
        cudaMalloc(&d_cnt, nb) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_code); cudaFree(d_cnt);
        return COV_ENOMEM;
    }
    auto done = [&](int r) { cudaFree(d_code); cudaFree(d_cnt); return r; };
    if (M > 0 && cudaMemcpy(d_code, code, (size_t)M * n, cudaMemcpyHostToDevice) != cudaSuccess) return done(-100);
    rc = cov_count_dev(q, n, R, d_code, M, d_cnt, nullptr);
    if (rc) return done(rc);
    std::vector<uint16_t> tmp;
    uint16_t *h = cnt;
    if (!h) { tmp.resize(g.N); h = tmp.data(); }
    cudaError_t e = cudaMemcpy(h, d_cnt, (size_t)g.N * 2, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return done(-(100 + (int)e));
    if (uncovered) {
        int64_t u = 0;
        for (uint32_t x = 0; x < g.N; x++) u += h[x] == 0;
        *uncovered = u;
    }
    return done(COV_OK);
}

}  // extern "C"
