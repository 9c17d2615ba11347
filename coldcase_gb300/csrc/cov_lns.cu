// cov_lns.cu -- GB300 (sm_103a) primitives of the transform-engine LNS
// (cov/gemm2/gpuchain.py, Engine; the reference's primitives are
// cov/gemm2/dct.cu behind cov/gemm2/dctlib.py).
//
// One cell (q, n, R) is resident on the device: the coverage multiplicity
// cnt[x] of the current code and an int32 map over all q^n words.  The maps
// the search reads are exact ball sums of an indicator:
//     gain(x) = #{y : d(x,y) <= R, cnt[y] == 0}   (newly covered by a codeword at x)
//     loss(x) = #{y : d(x,y) <= R, cnt[y] == 1}   (private words of a codeword at x)
// computed for every x by layers L_d[x] = #{marked y : d(x,y) = d}, d <= R,
// built one axis at a time: along an axis line of q words with layer sums
// S_d, a word's L_d gains S_{d-1} - L_{d-1}[x] (the marked words that now
// differ from it in this coordinate too).  After all n axes the map is
// sum_d L_d.  The same layers with the code itself marked give cnt.
//
// Words are indexed MSB-first (x = sum_j w_j q^(n-1-j)), as everywhere in
// this library.  Extraction returns positions in increasing index order, so
// every result is deterministic.
#include <cstdio>
#include <climits>
#include <cstring>
#include <vector>
#include <algorithm>
#include "cov_common.cuh"
#include "cov_tiles.cuh"
#include "../../include/covgpu.h"

#define LNS_MAXR 8
#define LNS_NT 256

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "covgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    return -(100 + (int)e_); } } while (0)

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
    void *scratch = nullptr;        // small device buffers of the calls
    size_t scratch_bytes = 0;
    unsigned long long *d_red = nullptr;
};

namespace {

struct LayerPtrs { int32_t *a[LNS_MAXR + 1]; };
struct LnsPw { uint32_t pw[COV_MAXN]; };

// indicator layer 0 from cnt: target 0 (uncovered) or 1 (private)
__global__ void k_lns_init(LayerPtrs L, int R1, const uint16_t *cnt, int target, uint32_t N)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) {
        L.a[0][x] = cnt[x] == target;
        for (int d = 1; d < R1; d++) L.a[d][x] = 0;
    }
}

// layer 0 = the code's words (each once per occurrence)
__global__ void k_lns_clear(LayerPtrs L, int R1, uint32_t N)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        for (int d = 0; d < R1; d++) L.a[d][x] = 0;
}

__global__ void k_lns_scatter(int32_t *A0, const uint32_t *idx, int m)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) atomicAdd(&A0[idx[i]], 1);
}

// One axis of stride s (s = q^k in the index): every line of q words
// x = hi*q*s + a*s + lo.  The layer sums of the line are read first; then,
// from the top layer down (so that layer d-1 is still the old one), each
// word's L_d gains S_{d-1} - L_{d-1}[x].  With `fin` (the last axis) the sum
// of the new layers goes to out (int32) or, saturated, to cnt16.
__global__ void k_lns_axis(LayerPtrs L, int R1, int q, uint32_t s, uint32_t nlines, int fin,
                           int32_t *out, uint16_t *cnt16)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nlines; f += gridDim.x * blockDim.x) {
        const uint32_t hi = f / s, lo = f - hi * s;
        const uint32_t base = hi * s * (uint32_t)q + lo;
        int32_t S[LNS_MAXR + 1];
        for (int d = 0; d < R1; d++) S[d] = 0;
        for (int a = 0; a < q; a++) {
            const uint32_t x = base + (uint32_t)a * s;
            for (int d = 0; d < R1 - 1; d++) S[d] += L.a[d][x];
        }
        for (int a = 0; a < q; a++) {
            const uint32_t x = base + (uint32_t)a * s;
            int32_t sum = L.a[0][x];
            int32_t below = sum;                      // old L_{d-1}[x]
            for (int d = 1; d < R1; d++) {
                const int32_t old = L.a[d][x];
                const int32_t nv = old + S[d - 1] - below;
                below = old;
                if (!fin) L.a[d][x] = nv;
                sum += nv;
            }
            if (fin) {
                if (out) out[x] = sum;
                else cnt16[x] = (uint16_t)min(sum, 65535);
            }
        }
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
__global__ void k_lns_hist(const int32_t *A, uint32_t N, int nbins, int vmax, unsigned long long *hist)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) {
        const int v = A[x];
        if (v < 1) continue;
        int b = (int)((long long)(min(v, vmax) - 1) * nbins / vmax);
        atomicAdd(&hist[b], 1ull);
    }
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

// One CTA per listed word: the ball's words, group by group (last position
// runs over its q-1 values).  op 0: count cnt == target (out[i]);
// op 1: add delta to cnt (saturating at 0 and 65535).
__global__ void k_lns_ball(uint16_t *cnt, const uint32_t *idx, int k, int q, int n, LnsPw g,
                           const uint64_t *items, const uint8_t *last, uint32_t ngroups, int op, int target,
                           int delta, int32_t *out)
{
    const int i = blockIdx.x;
    if (i >= k) return;
    const uint32_t base = idx[i];
    const uint64_t pc = lns_pack(base, q, n);
    int c = 0;
    for (uint32_t it = threadIdx.x; it < ngroups; it += blockDim.x) {
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
            if (op == 0) c += cnt[off] == target;
            else {
                const int v = (int)cnt[off] + delta;
                cnt[off] = (uint16_t)min(max(v, 0), 65535);
            }
        } else {
            const int step = (int)g.pw[lj], cj = cov_nib(pc, lj);
            int o2 = off - cj * step;
            for (int v = 0; v < q; v++, o2 += step) {
                if (v == cj) continue;
                if (op == 0) c += cnt[o2] == target;
                else {
                    const int nv = (int)cnt[o2] + delta;
                    cnt[o2] = (uint16_t)min(max(nv, 0), 65535);
                }
            }
        }
    }
    if (op == 0) {
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

int grid_of(uint32_t N)
{
    return (int)std::min<uint32_t>((N + LNS_NT - 1) / LNS_NT, (uint32_t)std::max(1, cov_sm_count()) * 8);
}

// the n axis passes over the layers; the last writes out or cnt16
int lns_passes(cov_lns *h, int32_t *out, uint16_t *cnt16)
{
    LayerPtrs L;
    for (int d = 0; d <= h->R; d++) L.a[d] = h->layer[d];
    const uint32_t nlines = h->N / (uint32_t)h->q;
    if (h->R == 0) {
        // no axis changes layer 0: the map is the indicator itself
        k_lns_axis<<<grid_of(nlines), LNS_NT>>>(L, 1, h->q, 1u, nlines, 1, out, cnt16);
        CK(cudaGetLastError());
        return 0;
    }
    for (int k = 0; k < h->n; k++) {
        const uint32_t s = h->pw[h->n - 1 - k];        // q^k
        k_lns_axis<<<grid_of(nlines), LNS_NT>>>(L, h->R + 1, h->q, s, nlines, k == h->n - 1, out, cnt16);
        CK(cudaGetLastError());
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
              cudaMalloc(&h->d_red, 64 * 8) == cudaSuccess;
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
    for (int d = 0; d <= LNS_MAXR; d++) cudaFree(h->layer[d]);
    cudaFree(h->scratch);
    delete h;
    return COV_OK;
}

int cov_lns_recount(cov_lns *h, const uint32_t *idx, int32_t m)
{
    if (!h || m < 0 || (m > 0 && !idx)) return COV_EINVAL;
    for (int i = 0; i < m; i++) if (idx[i] >= h->N) return COV_EINVAL;
    LayerPtrs L;
    for (int d = 0; d <= h->R; d++) L.a[d] = h->layer[d];
    k_lns_clear<<<grid_of(h->N), LNS_NT>>>(L, h->R + 1, h->N);
    CK(cudaGetLastError());
    if (m > 0) {
        int rc = lns_scratch(h, (size_t)m * 4);
        if (rc) return rc;
        CK(cudaMemcpy(h->scratch, idx, (size_t)m * 4, cudaMemcpyHostToDevice));
        k_lns_scatter<<<(m + 255) / 256, 256>>>(h->layer[0], (const uint32_t *)h->scratch, m);
        CK(cudaGetLastError());
    }
    int rc = lns_passes(h, nullptr, h->cnt);
    if (rc) return rc;
    CK(cudaDeviceSynchronize());
    return COV_OK;
}

int cov_lns_map(cov_lns *h, int32_t target)
{
    if (!h || target < 0) return COV_EINVAL;
    LayerPtrs L;
    for (int d = 0; d <= h->R; d++) L.a[d] = h->layer[d];
    k_lns_init<<<grid_of(h->N), LNS_NT>>>(L, h->R + 1, h->cnt, target, h->N);
    CK(cudaGetLastError());
    int rc = lns_passes(h, h->map, nullptr);
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
    if (!h || !hist || nbins < 1 || vmax < 1) return COV_EINVAL;
    int rc = lns_scratch(h, (size_t)nbins * 8);
    if (rc) return rc;
    unsigned long long *d_h = (unsigned long long *)h->scratch;
    CK(cudaMemset(d_h, 0, (size_t)nbins * 8));
    k_lns_hist<<<grid_of(h->N), LNS_NT>>>(h->map, h->N, nbins, vmax, d_h);
    CK(cudaGetLastError());
    CK(cudaMemcpy(hist, d_h, (size_t)nbins * 8, cudaMemcpyDeviceToHost));
    return COV_OK;
}

int cov_lns_map_extract(cov_lns *h, int32_t thr, int64_t cap, uint32_t *idx, int32_t *val, int64_t *found)
{
    if (!h || cap < 0 || (cap > 0 && (!idx || !val)) || !found) return COV_EINVAL;
    const uint32_t chunk = 65536;
    const uint32_t nb = (h->N + chunk - 1) / chunk;
    int rc = lns_scratch(h, (size_t)nb * 8 + (size_t)cap * 8 + 16);
    if (rc) return rc;
    uint32_t *bcount = (uint32_t *)h->scratch, *boff = bcount + nb;
    uint32_t *oidx = boff + nb;
    int32_t *oval = (int32_t *)(oidx + cap);
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
    const size_t k = (size_t)std::min<unsigned long long>(tot, (unsigned long long)cap);
    CK(cudaMemcpy(idx, oidx, k * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(val, oval, k * 4, cudaMemcpyDeviceToHost));
    return COV_OK;
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

int cov_lns_ball(cov_lns *h, const uint32_t *idx, int32_t k, int32_t op, int32_t arg, int32_t *out)
{
    if (!h || k < 0 || (k > 0 && !idx) || op < 0 || op > 1 || (op == 0 && k > 0 && !out)) return COV_EINVAL;
    if (k == 0) return COV_OK;
    for (int i = 0; i < k; i++) if (idx[i] >= h->N) return COV_EINVAL;
    int rc = lns_scratch(h, (size_t)k * 8);
    if (rc) return rc;
    uint32_t *d_i = (uint32_t *)h->scratch;
    int32_t *d_o = (int32_t *)(d_i + k);
    CK(cudaMemcpy(d_i, idx, (size_t)k * 4, cudaMemcpyHostToDevice));
    LnsPw g;
    memset(&g, 0, sizeof g);
    for (int j = 0; j < h->n; j++) g.pw[j] = h->pw[j];
    if (op == 0) {
        k_lns_ball<<<k, LNS_NT>>>(h->cnt, d_i, k, h->q, h->n, g, h->ball, h->ball_last, h->ngroups, 0, arg, 0,
                                  d_o);
        CK(cudaGetLastError());
        CK(cudaMemcpy(out, d_o, (size_t)k * 4, cudaMemcpyDeviceToHost));
    } else {
        // one word at a time: two balls may share words
        for (int i = 0; i < k; i++) {
            k_lns_ball<<<1, LNS_NT>>>(h->cnt, d_i + i, 1, h->q, h->n, g, h->ball, h->ball_last, h->ngroups, 1,
                                      0, arg, nullptr);
            CK(cudaGetLastError());
        }
        CK(cudaDeviceSynchronize());
    }
    return COV_OK;
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
