// cov_common.cuh -- device-side data layout and helpers shared by the
// covering-code search kernels (cov_engine.cu) and the verification kernels
// (cov_verify.cu).
//
// Word indexing follows the reference: x = sum_j w_j q^(n-1-j), MSB first
// (cov/engine/covsearch2e.c:916-921).  On the device a codeword is a packed
// uint64 with digit j in bits [4j, 4j+4) ("nibble j"), so q <= 16, n <= 16.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define COV_MAXN 16
#define COV_MAXQ 16

// ---------------------------------------------------------------- RNG ----
// xoshiro256++ seeded by four splitmix64 draws: the single stream that
// defines the search trajectory (cov/engine/covsearch2e.c:201-220).
struct CovRng { uint64_t s[4]; };

__host__ __device__ __forceinline__ uint64_t cov_rotl(uint64_t x, int k)
{
    return (x << k) | (x >> (64 - k));
}

__host__ __device__ __forceinline__ uint64_t cov_rng_next(CovRng &r)
{
    uint64_t out = cov_rotl(r.s[0] + r.s[3], 23) + r.s[0];
    uint64_t t = r.s[1] << 17;
    r.s[2] ^= r.s[0];
    r.s[3] ^= r.s[1];
    r.s[1] ^= r.s[2];
    r.s[0] ^= r.s[3];
    r.s[2] ^= t;
    r.s[3] = cov_rotl(r.s[3], 45);
    return out;
}

__host__ __device__ inline void cov_rng_seed(CovRng &r, uint64_t seed)
{
    for (int i = 0; i < 4; i++) {
        seed += 0x9E3779B97F4A7C15ULL;
        uint64_t z = seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        r.s[i] = z ^ (z >> 31);
    }
}

// ------------------------------------------------------- packed words ----
__host__ __device__ __forceinline__ int cov_nib(uint64_t pk, int j)
{
    return (int)((pk >> (4 * j)) & 15u);
}
__host__ __device__ __forceinline__ uint64_t cov_setnib(uint64_t pk, int j, int v)
{
    return (pk & ~(15ull << (4 * j))) | ((uint64_t)v << (4 * j));
}
// bit 4j set iff nibble j of x is nonzero: the difference set D(a,b) of
// two packed words is cov_spread(a ^ b), |D| its popcount.
__host__ __device__ __forceinline__ uint64_t cov_spread(uint64_t x)
{
    return (x | (x >> 1) | (x >> 2) | (x >> 3)) & 0x1111111111111111ull;
}
__device__ __forceinline__ int cov_dist(uint64_t a, uint64_t b)
{
    return __popcll(cov_spread(a ^ b));
}

// Counter word of the coverage array: the multiplicity in bits 0-15 and the
// sum (mod 2^16) of the ids of the covering codewords in bits 16-31.  When
// the multiplicity is 1 the sum is the id of the only covering codeword.
// Adding or removing coverer i is one 32-bit add of cov_cw_unit(i): the
// multiplicity never exceeds M <= 65535, so it never carries into the sum,
// and it is >= 1 before a removal, so nothing borrows from the sum.
__host__ __device__ __forceinline__ uint32_t cov_cw_unit(int i)
{
    return 1u + ((uint32_t)i << 16);
}

// ------------------------------------------------------------ slots ------
// One search instance.  Immutable after creation except through the
// pointed-to device arrays.
struct CovSlot {
    int q, n, R, M;
    uint32_t N;                  // q^n
    uint32_t pw[COV_MAXN];       // q^(n-1-j)
    int rs;                      // max(R,1): row stride of subset tables
    int nsub;                    // C(n-1,R): R-subsets avoiding one position
    int nfsub;                   // C(n,R)
    uint32_t ppow[COV_MAXN + 1]; // (q-1)^k
    int tenure, kick, cand;
    long long stall;
    long long neg_cluster_pairs; // list x candidate pairs above which the cluster shares the list pass
    int padj_warp;               // private-count events of a commit aggregated per warp
    int list_cost;               // cost of one list entry in walked words: the entering side
                                 // reads the list while U_n * list_cost < ncw (R+1) S
    int wide;                    // --wide: every single-coordinate move of a candidate codeword
                                 // while the list is valid and U_n n < (R+1) S'
    int wide_sliced;             // its list pass finds hits by bit-sliced counts (<= 64 candidates)
    int fix0;                    // --fix0: codeword 0 translated to 0^n and never moved (0 or 1)
    int sa;                      // --sa: focused simulated annealing instead of the tabu selection
    int noise;                   // --noise: per-mille of moves taken without evaluation
    double sa_t0, sa_cool, sa_tmin;  // --t0 --cool --tmin
    // device arrays
    uint32_t *cw;                // [N]  cnt (bits 0-15) | sum of covering ids mod 2^16 (16-31)
    uint64_t *code;              // [M]  packed codewords
    uint64_t *best;              // [M]  best code so far
    int32_t *tabu;               // [M*n*q]
    int32_t *P;                  // [M*(n+1)]: T_k, H_k[0..n-1]
    uint32_t *ul_idx;            // [ul_cap] uncovered-list word indices
    uint64_t *ul_pk;             // [ul_cap] their packed digits
    uint32_t *ul_bit;            // [ceil(N/32)] list membership
    uint32_t *zb;                // [ceil(N/32)] bit x set iff cnt[x] == 0 (kept when zbits)
    int zbits;                   // dense coverage: the entering walk reads zb, not the counts
    int ul_cap;
    const uint8_t *sub;          // [n][nsub][rs]
    const uint8_t *sub1;         // [n][nsub1][rs]: (R-1)-subsets avoiding one position
    int nsub1;                   // C(n-1,R-1)
    const uint8_t *ball_sub;     // concatenated r-subset tables, r = 0..R
    int ball_off[COV_MAXN + 2];  // start (in subsets) of radius r in ball_sub
    // state build by tiles: a tile is the q^bt_nl words that share their
    // first bt_nh digits; bt_items / bt_last list the ball of radius
    // <= min(R, bt_nl) on the low digits as groups (cov_tiles.cuh), by
    // radius: bt_v[r] groups have radius <= r
    const uint64_t *bt_items;
    const uint8_t *bt_last;
    int bt_nh, bt_nl;
    uint32_t bt_tw;              // q^bt_nl
    uint32_t bt_v[COV_MAXN + 2];
    // per-slot global scratch for the rare large cases
    uint32_t *g_perm;            // [M*n], [M*n*(q-1)] when wide
    int32_t *g_dval;             // same
    uint32_t *g_list;            // [M]
    int32_t *g_neg;              // [M*n]
    int32_t *g_negw;             // [M*n*q] entering counts of every move (wide only)
    void *trace;                 // cov_move_rec[trace_cap] or null
    long long trace_cap;
    struct CovSlotState *st;
};

// Mutable scalars of one instance, persisted between launches.
struct CovSlotState {
    uint64_t rng[4];
    long long it;                // iterations made so far
    long long unc;               // current uncovered count
    long long best_unc;
    long long since_improve;
    long long nkicks;
    long long trace_n;           // records written
    long long moves_left;        // budget of the current launch
    long long target;            // stop when best_unc <= target (-1: none)
    int ul_n;
    int ul_valid;
    int status;                  // 0 ok, negative = COV_E*
    int finished;                // 1 once uncovered reached 0
    long long stat_ul_pairs;     // uncovered-list x candidate-codeword pairs tested
    long long stat_commit_words;
    // cycle counts of the leader's phases, accumulated over launches:
    // 0 pick, 1 candidates + sample, 2 entering side, 3 select, 4 move op
    // (commit + sphere), 5 finish, 6 list compaction, 7 other ops
    long long it_limit;          // iteration count at which the slot stops (-1: none)
    double sa_T;                 // --sa: the temperature
    unsigned long long prof[24];   // 8..19: sub-phases (diagnostics: 11 RNG refill in the move op,
                                   // 12 wait for helper CTAs, 15 move op up to that wait); 20: sum of candidate
                                   // codewords, 21: sum of list lengths, 22: planned moves
};

// Generic enumeration unit of a sphere of radius r >= 1 around a word:
// one r-subset of positions and one assignment of non-centre values to its
// first r-1 positions; the q-1 values of the last position are the inner
// loop.  (The reference's odometer, covsearch2e.c:412-443, last digit
// fastest.)
struct CovItem {
    uint32_t w;      // word index with the last position still at the centre
    uint64_t pk;     // packed digits, same convention
    int last;        // last position of the subset
    int clast;       // centre digit there
    const uint8_t *ps;
};

__device__ __forceinline__ CovItem cov_item(const CovSlot &d, const uint8_t *subs, int r,
                                            uint32_t t, uint32_t base, uint64_t pc)
{
    CovItem it;
    const uint32_t pp = d.ppow[r - 1];
    const uint32_t s = t / pp;
    uint32_t rem = t - s * pp;
    const uint8_t *ps = subs + (size_t)s * d.rs;
    uint32_t w = base;
    uint64_t pk = pc;
    const int qm1 = d.q - 1;
    for (int k = r - 2; k >= 0; --k) {
        int dig = (int)(rem % (uint32_t)qm1);
        rem /= (uint32_t)qm1;
        int j = ps[k];
        int c = cov_nib(pc, j);
        int val = dig + (dig >= c);
        w += (uint32_t)((long long)(val - c) * (long long)d.pw[j]);
        pk = cov_setnib(pk, j, val);
    }
    it.w = w;
    it.pk = pk;
    it.last = ps[r - 1];
    it.clast = cov_nib(pc, it.last);
    it.ps = ps;
    return it;
}

// word of the inner loop: value index kk in [0, q-2] at the last position
__device__ __forceinline__ void cov_item_word(const CovSlot &d, const CovItem &it, int kk,
                                              uint32_t &w, uint64_t &pk)
{
    int val = kk + (kk >= it.clast);
    w = it.w + (uint32_t)((long long)(val - it.clast) * (long long)d.pw[it.last]);
    pk = cov_setnib(it.pk, it.last, val);
}

// ------------------------------------------------------ per device, host --
// Host-side facts that belong to one device: its SM count, and whether a
// kernel's attributes (the dynamic shared-memory opt-in, which
// cudaFuncSetAttribute sets for the current device only) were set on it.
#define COV_MAX_DEVICES 64

// SM count of the current device, cached per device (0 on error)
static inline int cov_sm_count()
{
    static int cache[COV_MAX_DEVICES];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 0;
    if (dev < COV_MAX_DEVICES && cache[dev]) return cache[dev];
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (dev < COV_MAX_DEVICES) cache[dev] = v;
    return v;
}

// One bit per device: set once a set-up step ran with that device current.
struct CovDeviceFlags {
    unsigned long long bits = 0;
    // true when the current device's bit is set; dev receives the device
    bool done(int &dev) const
    {
        dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= COV_MAX_DEVICES) return false;
        return (bits >> dev) & 1ull;
    }
    void set(int dev) { if (dev >= 0 && dev < COV_MAX_DEVICES) bits |= 1ull << dev; }
};

// L2-coherent global accessors: data written by other CTAs of the same
// launch is read with ld.global.cg so that no stale L1 line is observed.
template <class T>
__device__ __forceinline__ T cov_ldcg(const T *p) { return __ldcg(p); }
template <class T>
__device__ __forceinline__ void cov_stcg(T *p, T v) { __stcg(p, v); }
