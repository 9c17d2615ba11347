// cov_engine.cu -- GB300 (sm_103a) tabu engine for q-ary covering codes.
//
// The search is the reference engine's p5b trajectory
// (cov/engine/covsearch2e.c:1304-1580, `--preset p5b`, no --wide): the same
// RNG stream, candidate order, tie-breaking, tabu and kick rules, so every
// committed move and every delta equals the reference's.  What differs is how
// a move's delta is obtained:
//
//   * the reference walks, for every candidate codeword c, the whole
//     distance-R sphere around c to count T = #{w : d(w,c)=R, cnt[w]=1} and
//     H_j (covsearch2e.c:592-654), i.e. C(n,R)(q-1)^R gathers per candidate;
//   * here those counts are kept per codeword in P[k] = (T_k, H_k[0..n-1])
//     and updated incrementally: a word's count crosses 1 only inside a
//     commit or a kick, and when cnt[w] == 1 the covering codeword is named
//     by the sum of covering ids stored beside cnt.  Only the moved
//     codeword's sphere is walked again.  pos_p = T_k - H_k[p] exactly as in
//     covsearch2e.c:755-758.
//   * the entering side (neg) is read off the uncovered-word list as in
//     covsearch2e.c:720-734, or by the per-position walk of :735-753,
//     whichever costs less (the list while it is valid and short enough).
//
// Execution: one thread-block cluster per search instance ("slot").  The
// leader CTA (rank 0) runs the serial, RNG-ordered part of each iteration;
// every CTA of the cluster shares the commit and the sphere walks.  Plan and
// reductions travel through distributed shared memory; the CTAs meet at
// hardware cluster barriers, so there is no software spin-wait anywhere in
// the engine.  Each launch is bounded by a move budget, an op-count guard and
// a deadline counted in SM clock cycles.
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cooperative_groups.h>
#include "cov_common.cuh"
#include "cov_tiles.cuh"
#include "../../include/covgpu.h"

namespace cg = cooperative_groups;

#define NT        512          // threads per CTA
#define NWARP     (NT / 32)
#define PERM_CAP  2048         // candidates kept in shared memory
#define L_SM      128          // candidate codewords kept in shared memory
#define RB        1024         // scratch draws (FY chunk)
#define ULS       1024         // uncovered-list entries staged per chunk
#define RS        1024         // RNG stream ring (draws generated ahead)
#define RS_CKI    128          // a generator checkpoint every RS_CKI draws
#define RS_NCK    16           // checkpoints kept (RS_NCK * RS_CKI > RS + RS_CKI)
static_assert(RS % RS_CKI == 0 && (RS & (RS - 1)) == 0 && (RS_CKI & (RS_CKI - 1)) == 0,
              "RNG ring: powers of two, whole checkpoint blocks");
#define INV_N     1024         // moduli with a reciprocal in shared memory
#define CODE_SM   2048         // codewords mirrored in every CTA's shared memory
#define NEG_CLUSTER_PAIRS 4096  // list x candidate pairs above which the whole cluster helps
#define LIST_COST 5             // one uncovered-list entry costs about five walked words
#define UL_CAP_DEFAULT (1 << 20)

enum { OP_STOP = 0, OP_MOVE, OP_NEGWALK, OP_BALL, OP_RECOMPUTE, OP_ZERO_TABU, OP_REBUILD_UL, OP_NEG };
enum {
    PH_PLAN = 0, PH_SELECT, PH_FINISH_MOVE, PH_KICK_START, PH_KICK_PICK, PH_KICK_RECOMP,
    PH_KICK_END, PH_KICK_DONE, PH_REBUILD_DONE, PH_GREEDY, PH_GREEDY_NEXT, PH_STOPPED, PH_SA_END
};
enum { MODE_SEARCH = 0, MODE_GREEDY = 1 };

// Parameters of the op the leader broadcasts to the cluster.
struct OpParams {
    int op;
    int mi, mp, mv;            // codeword, position, value
    int sgn;                   // BALL: +1 / -1
    int ul_valid;
    uint32_t base, dv, basen;  // word index before / offset / after
    uint64_t pc, pcn, pu;      // packed codeword before / after, target word
    int nL, dtar;
    int L_sm, neg_sm;          // list / neg arrays live in the leader's smem
    int uln;                   // uncovered-list length for OP_NEG
    int wide;                  // OP_NEG counts every (candidate, position, value) into g_negw
};

// Sums of one op over the CTAs that share it: the change of the uncovered
// count and of the moved codeword's private counts T / H.
struct MoveAcc {
    unsigned long long dunc;
    int accT;
    int accH[COV_MAXN];
};

// One search instance's moves shared with helper CTAs outside its cluster
// (one instance on the whole GPU): the search cluster publishes each move
// here, the helpers take their share of its commit, add their sums to `acc`
// and count themselves in `done`.  Zeroed before every launch.
struct GridHelp {
    unsigned int seq;          // moves published in this launch
    unsigned int done;         // helper CTAs finished with the current move
    int stop;                  // the search cluster has left: helpers leave
    int code_gen;              // codeword changes other than moves (kicks) so far
    int absent;                // test setting: the helpers leave at once, so
                               // the leader's wait for them runs out
    int pad2;
    OpParams op;
    MoveAcc acc;
};

struct Smem {
    CovSlot slot;              // this CTA's copy of the slot descriptor
    OpParams opp;              // written by the leader
    OpParams opl;              // each CTA's local copy
    MoveAcc acc;               // leader accumulators (targets of DSMEM atomics)
    unsigned int gh_seq;       // moves published to the helpers (leader)
    int gh_got;                // helper: 1 a move to share, 0 leave
    double sa_T;               // --sa temperature
    int sa_p, sa_v;            // --sa: the proposed move of codeword L[0]
    int sa_accept;             // --sa: the proposal was accepted
    int noisy;                 // --noise: this move was taken without evaluation
    int code_cached;           // code_sm mirrors the code
    int code_gen;              // leader: codeword changes other than moves; helper: the last one seen
    int gh_reload;             // helper: reload code_sm before the move
    // per-CTA partials
    int partT;
    int partH[COV_MAXN];
    // leader state
    long long it, unc, best_unc, since_improve, nkicks, moves_left, target, trace_n;
    long long chosen_delta;
    unsigned long long t_deadline;
    long long guard;
    int ul_valid, status, phase, kick_t, finished, greedy_i, mode;
    int nL, dtar, ncand, take, improved, dokick, swaps_pending;
    int cpw, wide_now;         // candidate moves per codeword; --wide in force this move
    uint64_t pu;
    long long uw;
    cov_move_rec rec;
    unsigned long long prof[24];
    long long ul_pairs;
    int uln;                   // list length read once per iteration
    // scratch
    int red_i[NWARP];
    unsigned red_u[NWARP];
    unsigned long long red_ull[NWARP];
    int ibc[4];
    long long lbc[4];
    unsigned hitmask[2];
    // arrays
    uint32_t perm[PERM_CAP];
    int32_t dval[PERM_CAP];
    uint8_t tflag[PERM_CAP];
    int32_t fy_a[PERM_CAP];    // parallel Fisher-Yates scratch
    int32_t fy_b[PERM_CAP];
    int32_t fy_c[PERM_CAP];
    uint32_t L[L_SM];
    uint64_t Lpk[L_SM];
    int32_t neg[L_SM * COV_MAXN];
    uint32_t lbits[L_SM / 32];
    uint64_t cmask[COV_MAXN * COV_MAXQ]; // [j*q+v]: candidates (< 64) with digit v at position j
    uint16_t Pmask[L_SM];      // positions where candidate l differs from the sampled word
    uint64_t st_H[ULS];        // staged list chunk: candidates at distance R+1 from the entry
    uint16_t st_E[ULS];        //                    positions where the entry equals the sampled word
    uint64_t inv[INV_N + 1];   // floor((2^64-1)/m), m = 1..INV_N
    // RNG stream: draws generated ahead of use by an idle leader warp
    uint64_t rs_buf[RS];
    unsigned long long rs_gen, rs_use;
    CovRng rs_state;           // generator after rs_gen draws
    CovRng rs_ck[RS_NCK];      // generator at draw rs_ckpos[k]
    unsigned long long rs_ckpos[RS_NCK];
    uint64_t code_sm[CODE_SM]; // leader's mirror of the packed code (M <= CODE_SM)
    uint8_t dist8[CODE_SM];    // distances to the sampled word
};

static_assert(offsetof(Smem, fy_c) == offsetof(Smem, fy_a) + 2 * PERM_CAP * sizeof(int32_t),
              "the Fisher-Yates scratch doubles as one table during a move");

// ------------------------------------------------------------ helpers -----
__device__ __forceinline__ uint32_t widx_pk(const CovSlot &d, uint64_t pk)
{
    uint32_t x = 0;
    for (int j = 0; j < d.n; j++) x += (uint32_t)cov_nib(pk, j) * d.pw[j];
    return x;
}

__device__ __forceinline__ uint64_t pk_of_idx(const CovSlot &d, uint32_t x)
{
    uint64_t pk = 0;
    for (int j = d.n - 1; j >= 0; j--) {
        uint32_t qd = x / (uint32_t)d.q;
        pk |= (uint64_t)(x - qd * (uint32_t)d.q) << (4 * j);
        x = qd;
    }
    return pk;
}

__device__ __forceinline__ int cnt_of(const CovSlot &d, uint32_t w)
{
    return (int)(cov_ldcg(&d.cw[w]) & 0xffffu);
}

__device__ __forceinline__ int nth_set_pos(uint64_t spread, int r)
{
    for (int k = 0; k < r; k++) spread &= spread - 1;
    return (__ffsll((long long)spread) - 1) >> 2;
}

__device__ __forceinline__ uint64_t nibmask(int n)
{
    return n >= 16 ? 0x1111111111111111ull : (0x1111111111111111ull & ((1ull << (4 * n)) - 1));
}

__device__ __forceinline__ void set_error(const CovSlot &d, int code)
{
    atomicCAS(&d.st->status, 0, code);
}

// Block / cluster barriers that first reconverge the warp.  A lane held back
// on a divergent single-thread path (if (tid == 0) {...}) is otherwise
// scheduled long after its warp-mates have parked at the barrier; a warp
// barrier in front makes the scheduler run it at once.
__device__ __forceinline__ void cov_bar()
{
    __syncwarp();
    __syncthreads();
}
__device__ __forceinline__ int cov_bar_or(int v)
{
    __syncwarp();
    return __syncthreads_or(v);
}
__device__ __forceinline__ void cov_cbar(cg::cluster_group &cl)
{
    __syncwarp();
    cl.sync();
}

// cycle counter read that stays in program order with the memory operations
// around it (plain cov_clock() may be scheduled away from its position)
__device__ __forceinline__ long long cov_clock()
{
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t) :: "memory");
    return t;
}

// gpu-scope acquire load / release store of a 32-bit flag
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// The launch deadline is kept in SM cycles (read through cov_clock): a
// %globaltimer read can stall the reading warp for tens of microseconds,
// which is too slow for a check made every iteration.
#define COV_CYCLES_PER_NS 2ull

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sum of an int (all threads get the result)
__device__ int block_sum_int(Smem &S, int v)
{
    v = warp_sum(v);
    cov_bar();
    if ((threadIdx.x & 31) == 0) S.red_i[threadIdx.x >> 5] = v;
    cov_bar();
    int t = 0;
    for (int w = 0; w < NWARP; w++) t += S.red_i[w];
    cov_bar();
    return t;
}

__device__ unsigned block_min_u32(Smem &S, unsigned v)
{
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    cov_bar();
    if ((threadIdx.x & 31) == 0) S.red_u[threadIdx.x >> 5] = v;
    cov_bar();
    unsigned t = 0xffffffffu;
    for (int w = 0; w < NWARP; w++) t = min(t, S.red_u[w]);
    cov_bar();
    return t;
}

// exclusive prefix of flag over the block; returns the block total
__device__ int block_excl_scan(Smem &S, int flag, int &pos)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned m = __ballot_sync(0xffffffffu, flag);
    int inwarp = __popc(m & ((1u << lane) - 1));
    cov_bar();
    if (lane == 0) S.red_i[wid] = __popc(m);
    cov_bar();
    int before = 0, tot = 0;
    for (int w = 0; w < NWARP; w++) {
        if (w < wid) before += S.red_i[w];
        tot += S.red_i[w];
    }
    pos = before + inwarp;
    cov_bar();
    return tot;
}

// x mod m, exact: a shared-memory reciprocal for small m (at most two
// corrections), the generic 64-bit remainder otherwise
__device__ __forceinline__ uint64_t fastmod(const Smem &S, uint64_t x, uint64_t m)
{
    if (m <= INV_N) {
        uint64_t qe = __umul64hi(x, S.inv[m]);
        uint64_t r = x - qe * m;
        while (r >= m) r -= m;
        return r;
    }
    return x % m;
}

// ---- RNG stream.  The draws of the reference's single xoshiro256++ stream
// are consumed strictly in order; only how many each step consumes depends
// on the data.  So they are generated ahead into a ring (by the leader's
// warp 0 while the cluster works on a move) and consumed at a cursor; the
// generator state at the cursor is recovered from a checkpoint when the
// launch ends.  All rs_* calls are made by one thread.
__device__ __forceinline__ void rs_init(Smem &S, const uint64_t st[4])
{
    for (int k = 0; k < 4; k++) S.rs_state.s[k] = st[k];
    S.rs_gen = S.rs_use = 0;
    S.rs_ck[0] = S.rs_state;
    S.rs_ckpos[0] = 0;
    for (int k = 1; k < RS_NCK; k++) S.rs_ckpos[k] = ~0ull;
}

// generate until `limit` draws exist (never more than RS ahead of use)
__device__ __forceinline__ void rs_fill(Smem &S, unsigned long long limit)
{
    const unsigned long long cap = S.rs_use + RS;
    if (limit > cap) limit = cap;
    unsigned long long g = S.rs_gen;
    if (g >= limit) return;
    CovRng st = S.rs_state;
    while (g < limit) {
        if ((g & (RS_CKI - 1)) == 0) {
            const int k = (int)((g / RS_CKI) % RS_NCK);
            S.rs_ck[k] = st;
            S.rs_ckpos[k] = g;
        }
        // the draws up to the next checkpoint: RS is a multiple of RS_CKI,
        // so their ring slots are consecutive
        const unsigned long long nxt = min(limit, (g | (unsigned long long)(RS_CKI - 1)) + 1ull);
        uint64_t *buf = S.rs_buf + ((uint32_t)g & (RS - 1));
        const uint32_t cnt = (uint32_t)(nxt - g);
#pragma unroll 4
        for (uint32_t k = 0; k < cnt; k++) buf[k] = cov_rng_next(st);
        g = nxt;
    }
    S.rs_state = st;
    S.rs_gen = g;
}

__device__ __forceinline__ void rs_ensure(Smem &S, int need)
{
    if (S.rs_gen < S.rs_use + (unsigned long long)need) rs_fill(S, S.rs_use + (unsigned long long)need);
}

// k-th draw after the cursor (k < what rs_ensure secured)
__device__ __forceinline__ uint64_t rs_peek(const Smem &S, int k)
{
    return S.rs_buf[(S.rs_use + (unsigned long long)k) % RS];
}

__device__ __forceinline__ uint64_t rs_take(Smem &S)
{
    rs_ensure(S, 1);
    uint64_t v = S.rs_buf[S.rs_use % RS];
    S.rs_use++;
    return v;
}

// generator state positioned at the cursor
__device__ void rs_final(const Smem &S, uint64_t out[4])
{
    CovRng st;
    if (S.rs_gen == S.rs_use) {
        st = S.rs_state;
    } else {
        const unsigned long long blk = (S.rs_use / RS_CKI) * RS_CKI;
        const int k = (int)((S.rs_use / RS_CKI) % RS_NCK);
        st = S.rs_ck[k];
        for (unsigned long long g = blk; g < S.rs_use; g++) cov_rng_next(st);
    }
    for (int k = 0; k < 4; k++) out[k] = st.s[k];
}

__device__ __forceinline__ uint64_t leader_code(const CovSlot &d, const Smem &S, int i)
{
    return d.M <= CODE_SM ? S.code_sm[i] : cov_ldcg(&d.code[i]);
}

__device__ __forceinline__ void leader_set_code(const CovSlot &d, Smem &S, int i, uint64_t pk)
{
    cov_stcg(&d.code[i], pk);
    if (d.M <= CODE_SM) S.code_sm[i] = pk;
}

// exclusive scan of an int over the block with an associative op (applied
// in thread order); the block total goes to `total`
template <class Op>
__device__ int block_scan_int(Smem &S, int v, int ident, Op op, int &total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = op(y, x);
    }
    int ex = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) ex = ident;
    cov_bar();
    if (lane == 31) S.red_i[wid] = x;
    cov_bar();
    int pre = ident, tot = ident;
    for (int w = 0; w < NWARP; w++) {
        if (w < wid) pre = op(pre, S.red_i[w]);
        tot = op(tot, S.red_i[w]);
    }
    total = tot;
    cov_bar();
    return op(pre, ex);
}

// Fisher-Yates swaps of the sampled candidates (covsearch2e.c:1384-1389),
// their draws already reduced into dval[s] = j_s; one thread, in order (the
// oversized case; the shared-memory case is resolved by fy_parallel).
// Also counts the distinct codewords among the sample for the trace.
__device__ void apply_swaps(const CovSlot &d, Smem &S)
{
    if (!S.swaps_pending) return;
    const int take = S.take, ncand = S.ncand, cpw = S.cpw;
    const int psm = ncand <= PERM_CAP;
    uint32_t *perm = psm ? S.perm : d.g_perm;
    int32_t *dval = psm ? S.dval : d.g_dval;
    for (int s = 0; s < take; s++) {
        int j = dval[s];
        uint32_t tmp = perm[s]; perm[s] = perm[j]; perm[j] = tmp;
    }
    if (take < ncand) {
        int c = 0;
        for (int s = 0; s < take; s++) {
            int l = (int)(perm[s] / (uint32_t)cpw), dup = 0;
            for (int t = 0; t < s; t++) if ((int)(perm[t] / (uint32_t)cpw) == l) { dup = 1; break; }
            c += !dup;
        }
        S.rec.ncw = c;
    }
    S.swaps_pending = 0;
}

// ------------------------------------------------ private-count upkeep -----
// Word w (packed pkw) just became (s=+1) or stopped being (s=-1) privately
// covered by codeword k.  If w sits on k's distance-R sphere, T_k and H_k[j]
// (j in D(w,c_k)) move with it.
// During a move the adjustments collect in a per-CTA shared-memory table and
// reach P once per touched counter at the end of the move: early in a search
// about half of the 2 S' words of a commit cross multiplicity 1 <-> 2, and
// their coverers are few (those within 2R of the moved codeword), so
// adding each one to P in global memory serialises on a handful of rows.
// The table is indexed by codeword when M (n+1) counters fit, else a small
// open-addressing hash of rows; a row that finds no place goes to P directly.
#define PADJ_CAP (3 * PERM_CAP)    // int32 entries: the Fisher-Yates scratch, idle during a move
#define PADJ_PROBES 8
struct PAdjTab {
    int32_t *cnt;                  // rows of n+1 deltas
    int32_t *keys;                 // hashed form: codeword of each row (-1: free)
    int hs;                        // rows
    int w;                         // n + 1
    int direct;
};

__device__ __forceinline__ void private_adjust(const CovSlot &d, int k, uint64_t pkw, int s,
                                               const PAdjTab *t = nullptr)
{
    if (k < 0 || k >= d.M) { set_error(d, COV_EDRIFT); return; }
    extern __shared__ __align__(16) unsigned char cov_smem[];
    const Smem *Sm = reinterpret_cast<const Smem *>(cov_smem);
    const uint64_t ck = d.M <= CODE_SM && Sm->code_cached ? Sm->code_sm[k] : cov_ldcg(&d.code[k]);
    uint64_t D = cov_spread(pkw ^ ck);
    if (__popcll(D) != d.R) return;
    int32_t *Pk = nullptr;
    if (t) {
        if (t->direct) {
            Pk = t->cnt + k * t->w;
        } else {
            uint32_t h = ((uint32_t)k * 2654435761u) % (uint32_t)t->hs;
            for (int pr = 0; pr < PADJ_PROBES; pr++) {
                const int old = atomicCAS(&t->keys[h], -1, k);
                if (old == -1 || old == k) { Pk = t->cnt + h * t->w; break; }
                h = h + 1 == (uint32_t)t->hs ? 0 : h + 1;
            }
        }
    }
    if (!Pk) Pk = d.P + (size_t)k * (d.n + 1);
    atomicAdd(&Pk[0], s);
    while (D) {
        int j = (__ffsll((long long)D) - 1) >> 2;
        atomicAdd(&Pk[1 + j], s);
        D &= D - 1;
    }
}

// Warp-wide form for the commit: every lane of the warp calls it together;
// lane events (on) whose word lies on the distance-R sphere of codeword k
// (D = its difference set) are grouped by k, and one lane per group adds the
// group's counts -- neighbouring words of a commit mostly share their
// coverer, so per-lane atomics would queue on the same counters.
__device__ __forceinline__ void warp_private_adjust_slow(const CovSlot &d, const PAdjTab &t, bool ev, int k,
                                                      uint64_t pkw, int s)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    extern __shared__ __align__(16) unsigned char cov_smem[];
    uint64_t D = 0;
    bool on = false;
    if (ev) {
        if (k < 0 || k >= d.M) {
            set_error(d, COV_EDRIFT);
        } else {
            const Smem *Sm = reinterpret_cast<const Smem *>(cov_smem);
            const uint64_t ck = d.M <= CODE_SM && Sm->code_cached ? Sm->code_sm[k] : cov_ldcg(&d.code[k]);
            D = cov_spread(pkw ^ ck);
            on = __popcll(D) == d.R;
        }
    }
    const unsigned act = __ballot_sync(FULL, on);
    if (!act) return;
    const unsigned grp = __match_any_sync(FULL, on ? k : -1) & act;
    if (!__any_sync(FULL, on && grp != (1u << lane))) {
        // no two lanes share a coverer: each adds its own counts
        if (on) {
            int32_t *Pk = nullptr;
            if (t.direct) {
                Pk = t.cnt + k * t.w;
            } else {
                uint32_t h = ((uint32_t)k * 2654435761u) % (uint32_t)t.hs;
                for (int pr = 0; pr < PADJ_PROBES; pr++) {
                    const int old = atomicCAS(&t.keys[h], -1, k);
                    if (old == -1 || old == k) { Pk = t.cnt + h * t.w; break; }
                    h = h + 1 == (uint32_t)t.hs ? 0 : h + 1;
                }
                if (!Pk) Pk = d.P + (size_t)k * t.w;
            }
            atomicAdd(&Pk[0], s);
            uint64_t m = D;
            while (m) {
                const int j = (__ffsll((long long)m) - 1) >> 2;
                atomicAdd(&Pk[1 + j], s);
                m &= m - 1;
            }
        }
        return;
    }
    const bool lead = on && lane == __ffs(grp) - 1;
    int32_t *Pk = nullptr;
    if (lead) {
        if (t.direct) {
            Pk = t.cnt + k * t.w;
        } else {
            uint32_t h = ((uint32_t)k * 2654435761u) % (uint32_t)t.hs;
            for (int pr = 0; pr < PADJ_PROBES; pr++) {
                const int old = atomicCAS(&t.keys[h], -1, k);
                if (old == -1 || old == k) { Pk = t.cnt + h * t.w; break; }
                h = h + 1 == (uint32_t)t.hs ? 0 : h + 1;
            }
            if (!Pk) Pk = d.P + (size_t)k * t.w;
        }
        atomicAdd(&Pk[0], s * __popc(grp));
    }
    // positions present in any lane's difference set
    const unsigned ulo = __reduce_or_sync(FULL, (unsigned)D);
    const unsigned uhi = __reduce_or_sync(FULL, (unsigned)(D >> 32));
    uint64_t U = ((uint64_t)uhi << 32) | ulo;
    while (U) {
        const int j = (__ffsll((long long)U) - 1) >> 2;
        U &= U - 1;
        const unsigned b = __ballot_sync(FULL, on && ((D >> (4 * j)) & 1ull));
        if (lead) {
            const int c = __popc(b & grp);
            if (c) atomicAdd(&Pk[1 + j], s * c);
        }
    }
}

__device__ __forceinline__ void warp_private_adjust(const CovSlot &d, const PAdjTab &t, bool ev, int k,
                                                    uint64_t pkw, int s)
{
    if (__any_sync(0xffffffffu, ev)) warp_private_adjust_slow(d, t, ev, k, pkw, s);
}

__device__ __forceinline__ void ul_insert(const CovSlot &d, int ul_valid, uint32_t x, uint64_t pk)
{
    if (!ul_valid) return;
    uint32_t bit = 1u << (x & 31);
    uint32_t old = atomicOr(&d.ul_bit[x >> 5], bit);
    if (old & bit) return;
    int slot = atomicAdd(&d.st->ul_n, 1);
    if (slot < d.ul_cap) {
        cov_stcg(&d.ul_idx[slot], x);
        cov_stcg(&d.ul_pk[slot], pk);
    } else {
        atomicExch(&d.st->ul_n, d.ul_cap + 1);
    }
}

// the uncovered-word bitmap of dense slots, kept with every 0 <-> 1 crossing
__device__ __forceinline__ void zb_set(const CovSlot &d, uint32_t w)
{
    if (d.zbits) atomicOr(&d.zb[w >> 5], 1u << (w & 31));
}
__device__ __forceinline__ void zb_clear(const CovSlot &d, uint32_t w)
{
    if (d.zbits) atomicAnd(&d.zb[w >> 5], ~(1u << (w & 31)));
}

// word w loses coverage by codeword i (leaving side of a commit / -1 ball);
// o is the word's counter as loaded
__device__ __forceinline__ long long word_dec_v(const CovSlot &d, int ul_valid, int i, uint32_t w,
                                                uint64_t pk, uint32_t o, const PAdjTab *t = nullptr)
{
    uint32_t c = o & 0xffffu;
    if (c == 0) { set_error(d, COV_EDRIFT); return 0; }
    uint32_t nw = o - cov_cw_unit(i);
    cov_stcg(&d.cw[w], nw);
    if (c == 1) { ul_insert(d, ul_valid, w, pk); zb_set(d, w); return 1; }
    if (c == 2) private_adjust(d, (int)(nw >> 16), pk, +1, t);
    return 0;
}

// word w gains coverage by codeword i (entering side / +1 ball)
__device__ __forceinline__ long long word_inc_v(const CovSlot &d, int i, uint32_t w, uint64_t pk,
                                                uint32_t o, const PAdjTab *t = nullptr)
{
    uint32_t c = o & 0xffffu;
    if (c == 0xffffu) { set_error(d, COV_EDRIFT); return 0; }
    uint32_t nw = o + cov_cw_unit(i);
    cov_stcg(&d.cw[w], nw);
    if (c == 0) { zb_clear(d, w); return -1; }
    if (c == 1) private_adjust(d, (int)(o >> 16), pk, -1, t);
    return 0;
}

__device__ __forceinline__ long long word_dec(const CovSlot &d, int ul_valid, int i, uint32_t w, uint64_t pk)
{
    return word_dec_v(d, ul_valid, i, w, pk, cov_ldcg(&d.cw[w]));
}
__device__ __forceinline__ long long word_inc(const CovSlot &d, int i, uint32_t w, uint64_t pk)
{
    return word_inc_v(d, i, w, pk, cov_ldcg(&d.cw[w]));
}

// ------------------------------------------------------ cluster ops --------
__device__ __forceinline__ uint32_t sphere_items(const CovSlot &d, int r, int nsubs)
{
    return r == 0 ? 1u : (uint32_t)nsubs * d.ppow[r - 1];
}

// the CTA's share of a change in the uncovered count: reduced in the CTA,
// then one atomic into the leader's shared memory
__device__ __forceinline__ void cta_add_dunc(long long dunc, MoveAcc *acc)
{
    __shared__ long long cta_dunc;
    if (threadIdx.x == 0) cta_dunc = 0;
    __syncwarp();
    cov_bar();
    dunc = warp_sum(dunc);
    if ((threadIdx.x & 31) == 0 && dunc != 0) atomicAdd((unsigned long long *)&cta_dunc, (unsigned long long)dunc);
    cov_bar();
    if (threadIdx.x == 0 && cta_dunc != 0) atomicAdd(&acc->dunc, (unsigned long long)cta_dunc);
}

// add v to the shared counter of every position of a subset, once per group
// of lanes holding the same subset
__device__ __forceinline__ void group_add_h(int *partH, int key, int v, const uint8_t *ps, int r, int extra)
{
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, key);
    const int tot = __reduce_add_sync(grp, v);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1 && tot) {
        for (int s2 = 0; s2 < r; s2++) atomicAdd(&partH[ps[s2]], tot);
        if (extra >= 0) atomicAdd(&partH[extra], tot);
    }
}

// One move (i: p -> v) in a single pass over the cluster.
//  * Commit, covsearch2e.c:450-493 (mode 1) / 562-590: for every pattern
//    of R positions avoiding p, the leaving word a (d(a,c)=R, a_p=c_p) loses
//    codeword i and the entering word b = a + dv gains it.
//  * The private counts of i follow the move exactly without a new sphere
//    walk: d(w,c') = d(w,c) + [w_p == c_p] - [w_p == v], so only words with
//    w_p in {c_p, v} change sphere membership -- the leaving words (out),
//    the entering words (in), X = {w_p = v, d(w,c) = R} (out) and
//    Y = {w_p = c_p, d(w,c) = R-1} (in); X = Y + dv.  The counts of X and Y
//    are not changed by the move, so they are read in the same pass.
// The change of T_i / H_i goes to the leader's accT / accH.
// Leaving / entering pairs of a commit (covsearch2e.c:450-493): the S'
// patterns of R positions avoiding p, q-1 values of the last one per item.
// Per-lane form: each private-count event goes to P on its own.
__device__ __forceinline__ void commit_pairs_lane(const CovSlot &d, const OpParams &P, Smem &S, uint32_t wid,
                                               uint32_t wstride, int &T, long long &dunc)
{
    const int R = d.R, lane = threadIdx.x & 31;
    const uint8_t *subp = d.sub + (size_t)P.mp * d.nsub * d.rs;
    const uint32_t nit = (uint32_t)d.nsub * d.ppow[R - 1];
    const uint32_t nstep = (nit + 31) / 32 * 32;
    const int qm1 = d.q - 1;

        // few private-count events per move: each lane adds its own to P
    for (uint32_t t0 = wid * 32; t0 < nstep; t0 += wstride) {
        const uint32_t t = t0 + lane;
        int dt = 0;
        int key = -1;
        const uint8_t *ps = subp;
        if (t < nit) {
            // every word of the item is distinct: all 2(q-1) counters are
            // loaded before any is written, so the loads are in flight together
            CovItem it = cov_item(d, subp, R, t, P.base, P.pc);
            key = (int)(t / d.ppow[R - 1]);
            ps = it.ps;
            uint32_t oa[COV_MAXQ - 1], ob[COV_MAXQ - 1];
#pragma unroll
            for (int kk = 0; kk < COV_MAXQ - 1; kk++) {
                if (kk < qm1) {
                    uint32_t a; uint64_t pka;
                    cov_item_word(d, it, kk, a, pka);
                    oa[kk] = cov_ldcg(&d.cw[a]);
                    ob[kk] = cov_ldcg(&d.cw[a + P.dv]);
                }
            }
#pragma unroll
            for (int kk = 0; kk < COV_MAXQ - 1; kk++) {
                if (kk < qm1) {
                    uint32_t a; uint64_t pka;
                    cov_item_word(d, it, kk, a, pka);
                    dt -= (oa[kk] & 0xffffu) == 1;
                    dt += (ob[kk] & 0xffffu) == 0;
                    dunc += word_dec_v(d, P.ul_valid, P.mi, a, pka, oa[kk]);
                    dunc += word_inc_v(d, P.mi, a + P.dv, cov_setnib(pka, P.mp, P.mv), ob[kk]);
                }
            }
        }
        T += dt;
        if (t0 < nit) group_add_h(S.partH, key, dt, ps, R, -1);
    }
}

// Warp-aggregated form: events collected into the shared table.
__device__ __forceinline__ void commit_pairs_warp(const CovSlot &d, const OpParams &P, Smem &S, const PAdjTab &tab,
                                               uint32_t wid, uint32_t wstride, int &T, long long &dunc)
{
    const int R = d.R, lane = threadIdx.x & 31;
    const uint8_t *subp = d.sub + (size_t)P.mp * d.nsub * d.rs;
    const uint32_t nit = (uint32_t)d.nsub * d.ppow[R - 1];
    const uint32_t nstep = (nit + 31) / 32 * 32;
    const int qm1 = d.q - 1;

        // many events: collected per warp into the shared table
    const uint32_t unit = cov_cw_unit(P.mi);
    constexpr int CH = 8;
    for (uint32_t t0 = wid * 32; t0 < nstep; t0 += wstride) {
        const uint32_t t = t0 + lane;
        const bool live = t < nit;
        int dt = 0;
        int key = -1;
        const uint8_t *ps = subp;
        // every word of the item is distinct: all 2(q-1) counters are
        // loaded before any is written, so the loads are in flight together
        CovItem it = cov_item(d, subp, R, live ? t : 0, P.base, P.pc);
        if (live) {
            key = (int)(t / d.ppow[R - 1]);
            ps = it.ps;
        }
        // values of the last position in chunks of CH (one chunk for q <= 9)
        for (int kb = 0; kb < qm1; kb += CH) {
        uint32_t oa[CH], ob[CH];
        if (live) {
#pragma unroll
            for (int kc = 0; kc < CH; kc++) {
                if (kb + kc < qm1) {
                    uint32_t a; uint64_t pka;
                    cov_item_word(d, it, kb + kc, a, pka);
                    oa[kc] = cov_ldcg(&d.cw[a]);
                    ob[kc] = cov_ldcg(&d.cw[a + P.dv]);
                }
            }
        }
        // leaving word a loses codeword i, entering word a + dv gains it
        // (the steps of word_dec_v / word_inc_v, with the private-count
        // events handed to the warp-wide adjust)
#pragma unroll
        for (int kc = 0; kc < CH; kc++) {
            if (kb + kc < qm1) {
                bool evd = false, evi = false;
                int kd = 0, ki = 0;
                uint64_t pka = 0;
                if (live) {
                    uint32_t a;
                    cov_item_word(d, it, kb + kc, a, pka);
                    const uint32_t o1 = oa[kc], o2 = ob[kc];
                    const uint32_t c1 = o1 & 0xffffu, c2 = o2 & 0xffffu;
                    dt -= c1 == 1;
                    dt += c2 == 0;
                    if (c1 == 0 || c2 == 0xffffu) {
                        set_error(d, COV_EDRIFT);
                    } else {
                        const uint32_t n1 = o1 - unit;
                        cov_stcg(&d.cw[a], n1);
                        cov_stcg(&d.cw[a + P.dv], o2 + unit);
                        if (c1 == 1) { ul_insert(d, P.ul_valid, a, pka); zb_set(d, a); dunc += 1; }
                        else if (c1 == 2) { evd = true; kd = (int)(n1 >> 16); }
                        if (c2 == 0) { zb_clear(d, a + P.dv); dunc -= 1; }
                        else if (c2 == 1) { evi = true; ki = (int)(o2 >> 16); }
                    }
                }
                warp_private_adjust(d, tab, evd, kd, pka, +1);
                warp_private_adjust(d, tab, evi, ki, cov_setnib(pka, P.mp, P.mv), -1);
            }
        }
        }
        T += dt;
        if (t0 < nit) group_add_h(S.partH, key, dt, ps, R, -1);
    }
}

// part / parts: this CTA's share of the move among all CTAs that take one
// (the search cluster first, then any helper CTAs); acc receives the sums
// (the leader's shared memory, or the helpers' global accumulator).  With
// lead set the leader CTA (part 0) takes no share: its warp 0 generates the
// next draws of the RNG stream with the SM to itself, which with helper CTAs
// is the longest task of a move.
template <bool WARP>
__device__ __forceinline__ void op_move_t(const CovSlot &d, const OpParams &P, Smem &S, MoveAcc *acc, int part,
                                          int parts, bool lead = false)
{
    const int R = d.R, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) S.partT = 0;
    __syncwarp();
    if (threadIdx.x < COV_MAXN) S.partH[threadIdx.x] = 0;
    PAdjTab tab;
    tab.w = d.n + 1;
    tab.direct = d.M * tab.w <= PADJ_CAP;
    tab.hs = !WARP || R == 0 ? 0 : tab.direct ? d.M : PADJ_CAP / (tab.w + 1);
    tab.keys = S.fy_a;
    tab.cnt = tab.direct ? S.fy_a : S.fy_a + tab.hs;
    if (WARP) {
        const int nk = tab.direct ? 0 : tab.hs;
        const int ne = nk + tab.hs * tab.w;
        for (int e = threadIdx.x; e < ne; e += NT) S.fy_a[e] = e < nk ? -1 : 0;
    }
    cov_bar();
    long long dunc = 0;
    int T = 0;
    // the leader's warp 0 generates RNG draws for the next iterations while
    // every other warp of the cluster shares the move
    const int warp = (int)(threadIdx.x >> 5);
    // with lead the share of the CTAs is interleaved (warp-major), so that a
    // move with fewer items than warps spreads its gathers over every SM
    const int gw = !lead ? part * NWARP + warp - 1 : part == 0 ? (warp == 0 ? -1 : -2) : warp * (parts - 1) + part - 1;
    const uint32_t wid = (uint32_t)max(gw, 0);
    const uint32_t wstride = (uint32_t)(lead ? (parts - 1) * NWARP : parts * NWARP - 1) * 32;
    const int p0 = lead ? 1 : 0;                 // the part whose thread 32 takes the single-word steps
    if (gw < 0) {
        if (gw == -1 && threadIdx.x == 0) {
            const long long t0 = cov_clock();
            rs_fill(S, S.rs_use + RS);
            S.prof[11] += cov_clock() - t0;
        }
        __syncwarp();
    } else if (R == 0) {
        if (part == p0 && threadIdx.x == 32) {
            const uint32_t oa = cov_ldcg(&d.cw[P.base]);
            const uint32_t ob = cov_ldcg(&d.cw[P.base + P.dv]);
            T -= (oa & 0xffffu) == 1;
            T += (ob & 0xffffu) == 0;
            dunc += word_dec_v(d, P.ul_valid, P.mi, P.base, P.pc, oa);
            dunc += word_inc_v(d, P.mi, P.base + P.dv, P.pcn, ob);
        }
    } else {
        // leaving / entering pairs
        if (WARP) commit_pairs_warp(d, P, S, tab, wid, wstride, T, dunc);
        else commit_pairs_lane(d, P, S, wid, wstride, T, dunc);
        const int qm1 = d.q - 1;
        // X / Y pairs: (R-1)-subsets avoiding p
        if (R == 1) {
            if (part == p0 && threadIdx.x == 32) {
                const int dy = (int)((cov_ldcg(&d.cw[P.base]) & 0xffffu) == 1) -
                               (int)((cov_ldcg(&d.cw[P.base + P.dv]) & 0xffffu) == 1);
                T += dy;
                if (dy) atomicAdd(&S.partH[P.mp], dy);
            }
        } else {
            const uint8_t *subq = d.sub1 + (size_t)P.mp * d.nsub1 * d.rs;
            const uint32_t pq = d.ppow[R - 2];
            const uint32_t nxy = (uint32_t)d.nsub1 * pq;
            const uint32_t nstep2 = (nxy + 31) / 32 * 32;
            for (uint32_t t0 = wid * 32; t0 < nstep2; t0 += wstride) {
                const uint32_t t = t0 + lane;
                int dy = 0;
                int key = -1;
                const uint8_t *ps = subq;
                if (t < nxy) {
                    CovItem it = cov_item(d, subq, R - 1, t, P.base, P.pc);
                    key = (int)(t / pq);
                    ps = it.ps;
                    uint32_t cy[COV_MAXQ - 1], cx[COV_MAXQ - 1];
#pragma unroll
                    for (int kk = 0; kk < COV_MAXQ - 1; kk++) {
                        if (kk < qm1) {
                            uint32_t y; uint64_t pky;
                            cov_item_word(d, it, kk, y, pky);
                            cy[kk] = cov_ldcg(&d.cw[y]);
                            cx[kk] = cov_ldcg(&d.cw[y + P.dv]);
                        }
                    }
#pragma unroll
                    for (int kk = 0; kk < COV_MAXQ - 1; kk++)
                        if (kk < qm1) dy += (int)((cy[kk] & 0xffffu) == 1) - (int)((cx[kk] & 0xffffu) == 1);
                }
                T += dy;
                if (t0 < nxy) group_add_h(S.partH, key, dy, ps, R - 1, P.mp);
            }
        }
    }
    cta_add_dunc(dunc, acc);
    T = warp_sum(T);
    if (lane == 0 && T) atomicAdd(&S.partT, T);
    cov_bar();
    if (threadIdx.x == 0 && S.partT) atomicAdd(&acc->accT, S.partT);
    if (threadIdx.x < d.n && S.partH[threadIdx.x]) atomicAdd(&acc->accH[threadIdx.x], S.partH[threadIdx.x]);
    // private-count deltas of this CTA to P
    if (WARP) for (int e = threadIdx.x; e < tab.hs * tab.w; e += NT) {
        const int v = tab.cnt[e];
        if (!v) continue;
        const int row = e / tab.w;
        const int k = tab.direct ? row : tab.keys[row];
        atomicAdd(&d.P[(size_t)k * tab.w + (e - row * tab.w)], v);
    }
}

// T and H of the codeword with packed digits pc at word index base: one
// walk of its distance-R sphere (covsearch2e.c:621-650, read side only).
// Work unit: one R-subset and a block of 32 assignments of its first R-1
// positions, one per lane, so that the warp shares the subset and adds its
// count to the R position counters once.
__device__ void op_recompute(const CovSlot &d, uint32_t base, uint64_t pc, Smem &S, Smem *LS,
                             int rank, int csize)
{
    const int R = d.R;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) S.partT = 0;
    __syncwarp();
    if (threadIdx.x < COV_MAXN) S.partH[threadIdx.x] = 0;
    cov_bar();
    int T = 0;
    if (R == 0) {
        if (rank == 0 && threadIdx.x == 0) T = (cnt_of(d, base) == 1);
    } else {
        const uint8_t *fs = d.ball_sub + (size_t)d.ball_off[R] * d.rs;
        const uint32_t pp = d.ppow[R - 1];
        const uint32_t nblk = (pp + 31) / 32;
        const uint32_t units = (uint32_t)d.nfsub * nblk;
        const uint32_t gw = (uint32_t)rank * NWARP + (threadIdx.x >> 5);
        const uint32_t wstride = (uint32_t)csize * NWARP;
        for (uint32_t u = gw; u < units; u += wstride) {
            const uint32_t sub = u / nblk;
            const uint32_t r = (u - sub * nblk) * 32 + lane;
            int t1 = 0;
            if (r < pp) {
                CovItem it = cov_item(d, fs, R, sub * pp + r, base, pc);
                for (int kk = 0; kk < d.q - 1; kk++) {
                    uint32_t w; uint64_t pk;
                    cov_item_word(d, it, kk, w, pk);
                    t1 += (cnt_of(d, w) == 1);
                }
            }
            t1 = warp_sum(t1);
            if (lane == 0 && t1) {
                T += t1;
                const uint8_t *ps = fs + (size_t)sub * d.rs;
                for (int s2 = 0; s2 < R; s2++) atomicAdd(&S.partH[ps[s2]], t1);
            }
        }
    }
    if (lane == 0 && T) atomicAdd(&S.partT, T);
    cov_bar();
    if (threadIdx.x == 0 && S.partT) atomicAdd(&LS->acc.accT, S.partT);
    if (threadIdx.x < d.n && S.partH[threadIdx.x]) atomicAdd(&LS->acc.accH[threadIdx.x], S.partH[threadIdx.x]);
}

// +1 / -1 over the whole radius-R ball of codeword i: covsearch2e.c:353-380
__device__ void op_ball(const CovSlot &d, const OpParams &P, Smem *LS, int rank, int csize)
{
    const int R = d.R;
    uint32_t cum[COV_MAXN + 2];
    cum[0] = 1;   // the centre
    for (int r = 1; r <= R; r++)
        cum[r] = cum[r - 1] + sphere_items(d, r, d.ball_off[r + 1] - d.ball_off[r]);
    const uint32_t nit = cum[R];
    const uint32_t stride = (uint32_t)csize * NT;
    long long dunc = 0;
    for (uint32_t t = (uint32_t)rank * NT + threadIdx.x; t < nit; t += stride) {
        if (t == 0) {
            if (P.sgn < 0) dunc += word_dec(d, P.ul_valid, P.mi, P.base, P.pc);
            else dunc += word_inc(d, P.mi, P.base, P.pc);
            continue;
        }
        int r = 1;
        while (t >= cum[r]) r++;
        const uint8_t *subs = d.ball_sub + (size_t)d.ball_off[r] * d.rs;
        CovItem it = cov_item(d, subs, r, t - cum[r - 1], P.base, P.pc);
        for (int kk = 0; kk < d.q - 1; kk++) {
            uint32_t w; uint64_t pk;
            cov_item_word(d, it, kk, w, pk);
            if (P.sgn < 0) dunc += word_dec(d, P.ul_valid, P.mi, w, pk);
            else dunc += word_inc(d, P.mi, w, pk);
        }
    }
    cta_add_dunc(dunc, &LS->acc);
}

// Entering-side counts by walking, used while the uncovered list is not
// valid: covsearch2e.c:656-683, 735-753.
// CHUNK: the values of an item loaded together in chunks of 8 (faster; used
// by the engine instantiation for dense-coverage slots, whose register
// budget has room for it).
template <bool CHUNK>
__device__ void op_negwalk(const CovSlot &d, const OpParams &P, Smem &S, Smem *LS, int rank,
                           int csize, cg::cluster_group &cl)
{
    constexpr int WCH = 8;
    const int R = d.R;
    const uint32_t *Lp = P.L_sm ? cl.map_shared_rank(S.L, 0) : d.g_list;
    int32_t *negp = P.neg_sm ? cl.map_shared_rank(S.neg, 0) : d.g_neg;
    const uint32_t nit = sphere_items(d, R, d.nsub);
    const unsigned long long per_l = (unsigned long long)P.dtar * nit;
    const unsigned long long total = per_l * (unsigned long long)P.nL;
    const unsigned long long stride = (unsigned long long)csize * NT;
    // A thread's consecutive items mostly share their (candidate, position):
    // the item index advances incrementally and the candidate's codeword,
    // position and word base are recomputed only when those change.
    int l = -1, pi = 0, p = 0;
    uint32_t tt = 0, b0 = 0;
    uint64_t pc2 = 0;
    int cur_l = -1, cur_pi = -1;
    for (unsigned long long t = (unsigned long long)rank * NT + threadIdx.x; t < total; t += stride) {
        if (l < 0 || (unsigned long long)tt + stride >= nit) {
            l = (int)(t / per_l);
            const unsigned long long rem = t - (unsigned long long)l * per_l;
            pi = (int)(rem / nit);
            tt = (uint32_t)(rem - (unsigned long long)pi * nit);
        } else {
            tt += (uint32_t)stride;
        }
        if (l != cur_l || pi != cur_pi) {
            const int k = P.L_sm ? (int)Lp[l] : (int)cov_ldcg(&Lp[l]);
            const uint64_t pck = cov_ldcg(&d.code[k]);
            p = nth_set_pos(cov_spread(pck ^ P.pu), pi);
            const int v = cov_nib(P.pu, p), c = cov_nib(pck, p);
            b0 = widx_pk(d, pck) + (uint32_t)((long long)(v - c) * (long long)d.pw[p]);
            pc2 = cov_setnib(pck, p, v);
            cur_l = l;
            cur_pi = pi;
        }
        int nz = 0;
        if (R == 0) {
            nz = (cnt_of(d, b0) == 0);
        } else {
            const uint8_t *subp = d.sub + (size_t)p * d.nsub * d.rs;
            CovItem it = cov_item(d, subp, R, tt, b0, pc2);
            // loads of a chunk of values in flight together
            const int qm1 = d.q - 1;
            if (!CHUNK) {
                for (int kk = 0; kk < qm1; kk++) {
                    uint32_t w; uint64_t pk;
                    cov_item_word(d, it, kk, w, pk);
                    nz += (cnt_of(d, w) == 0);
                }
            } else if (d.zbits) {
                // dense coverage: one bit per word, the bitmap stays in L2.
                // The item's words rise by the last position's stride; a
                // bitmap word they share is loaded once.
                for (int kb = 0; kb < qm1; kb += WCH) {
                    uint32_t cv[WCH];
                    uint32_t prev = 0xffffffffu;
#pragma unroll
                    for (int kc = 0; kc < WCH; kc++) {
                        if (kb + kc < qm1) {
                            uint32_t w; uint64_t pk;
                            cov_item_word(d, it, kb + kc, w, pk);
                            if ((w >> 5) != prev) cv[kc] = cov_ldcg(&d.zb[w >> 5]);
                            prev = w >> 5;
                        }
                    }
                    prev = 0xffffffffu;
#pragma unroll
                    for (int kc = 0; kc < WCH; kc++) {
                        if (kb + kc < qm1) {
                            uint32_t w; uint64_t pk;
                            cov_item_word(d, it, kb + kc, w, pk);
                            if ((w >> 5) == prev) cv[kc] = cv[kc - 1];
                            prev = w >> 5;
                            nz += (int)((cv[kc] >> (w & 31)) & 1u);
                        }
                    }
                }
            } else for (int kb = 0; kb < qm1; kb += WCH) {
                uint32_t cv[WCH];
#pragma unroll
                for (int kc = 0; kc < WCH; kc++) {
                    if (kb + kc < qm1) {
                        uint32_t w; uint64_t pk;
                        cov_item_word(d, it, kb + kc, w, pk);
                        cv[kc] = cov_ldcg(&d.cw[w]);
                    }
                }
#pragma unroll
                for (int kc = 0; kc < WCH; kc++)
                    if (kb + kc < qm1) nz += (cv[kc] & 0xffffu) == 0;
            }
        }
        // lanes of a warp mostly walk the same (codeword, position): one
        // atomic per group
        const unsigned am = __activemask();
        const int key = l * d.n + p;
        const unsigned grp = __match_any_sync(am, key);
        const int sum = __reduce_add_sync(grp, nz);
        if ((threadIdx.x & 31) == __ffs(grp) - 1 && sum) atomicAdd(&negp[key], sum);
    }
}

__device__ void op_zero_tabu(const CovSlot &d, int rank, int csize)
{
    const size_t tot = (size_t)d.M * d.n * d.q;
    for (size_t x = (size_t)rank * NT + threadIdx.x; x < tot; x += (size_t)csize * NT)
        cov_stcg(&d.tabu[x], 0);
}

// rebuild of the uncovered list from cnt (covsearch2e.c:323-338): clear the
// membership bits, then append every zero-count word.
__device__ void op_rebuild_ul(const CovSlot &d, int rank, int csize, cg::cluster_group &cl)
{
    const uint32_t nb = (d.N + 31) / 32;
    for (uint32_t x = (uint32_t)rank * NT + threadIdx.x; x < nb; x += (uint32_t)csize * NT)
        cov_stcg(&d.ul_bit[x], 0u);
    cov_cbar(cl);
    for (uint32_t x = (uint32_t)rank * NT + threadIdx.x; x < d.N; x += (uint32_t)csize * NT) {
        if ((cov_ldcg(&d.cw[x]) & 0xffffu) == 0) ul_insert(d, 1, x, pk_of_idx(d, x));
    }
}

// Entering side from the uncovered-word list (covsearch2e.c:720-734) for
// more than 64 candidates (at most that many take neg_chunks): for every
// listed x that is still uncovered and every candidate codeword c with
// d(x,c) = R+1, neg[c][j] += 1 for each j in D(x,c) with x_j = u_j.
// Entries first, first+stride, ... of the list.
__device__ void ul_pass(const CovSlot &d, uint64_t pu, int nL, const uint64_t *Lpk, int32_t *negp,
                        uint32_t first, uint32_t stride, uint32_t n0)
{
    const int n = d.n, R = d.R;
    const uint64_t nm = nibmask(n);
    for (uint32_t e = first; e < n0; e += stride) {
        const uint32_t x = cov_ldcg(&d.ul_idx[e]);
        const uint64_t px = cov_ldcg(&d.ul_pk[e]);
        if ((cov_ldcg(&d.cw[x]) & 0xffffu) != 0) continue;     // stale entry
        const uint64_t eq = ~cov_spread(px ^ pu) & nm;
        for (int l = 0; l < nL; l++) {
            const uint64_t D = cov_spread(px ^ Lpk[l]);
            if (__popcll(D) != R + 1) continue;
            for (uint64_t m = D & eq; m; m &= m - 1)
                atomicAdd(&negp[l * n + ((__ffsll((long long)m) - 1) >> 2)], 1);
        }
    }
}

// The entering side for at most 64 candidates, without atomics.  The list
// entries [e0, e1) are taken in chunks of ULS, as groups of 32 (one per
// lane of a warp).  For each group a warp records, by ballot, which of its
// entries each candidate hits at distance R+1 (LM[l]) and which equal the
// sampled word u at each position (EJ[j]); stale entries (covered again) hit
// nothing.  For candidate l and a position j where c_l differs from u,
// neg[l][j] then gains popc(LM[l] & EJ[j]) over the groups: exactly the
// entries x with d(x,c_l) = R+1, j in D(x,c_l) and x_j = u_j.  Each thread
// owns fixed (l, j) pairs and keeps their sums in registers until the end.
// The masks live in st_H/st_E, rows XOR-swizzled by group so that threads
// reading different rows hit different banks.
__device__ void neg_chunks(const CovSlot &d, Smem &S, uint64_t pu, int nL, uint32_t e0, uint32_t e1,
                           int32_t *negp)
{
    const int n = d.n, q = d.q, R = d.R;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nm = nibmask(n);
    const int tgt = n - (R + 1);
    const uint64_t lmask = nL >= 64 ? ~0ull : ((1ull << nL) - 1);
    constexpr int NG = ULS / 32;                       // groups per chunk (32)
    uint32_t *LM = reinterpret_cast<uint32_t *>(S.st_H);   // [64][NG]
    uint32_t *EJ = reinterpret_cast<uint32_t *>(S.st_E);   // [16][NG]
    const int npair = nL * n;
    int acc0 = 0, acc1 = 0;                            // pairs threadIdx.x and threadIdx.x + NT
    for (uint32_t c0 = e0; c0 < e1; c0 += ULS) {
        const int cnt = (int)min((uint32_t)ULS, e1 - c0);
        const int ng = (cnt + 31) >> 5;
        for (int g = warp; g < ng; g += NWARP) {
            const int k = g * 32 + lane;
            const bool valid = k < cnt;
            uint64_t px = 0, hit = 0;
            if (valid) {
                px = cov_ldcg(&d.ul_pk[c0 + (uint32_t)k]);
                uint64_t b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0;
                for (int j = 0; j < n; j++) {
                    const uint64_t m = S.cmask[j * q + cov_nib(px, j)];
                    uint64_t c1 = b0 & m; b0 ^= m;
                    uint64_t c2 = b1 & c1; b1 ^= c1;
                    uint64_t c3 = b2 & c2; b2 ^= c2;
                    uint64_t c4 = b3 & c3; b3 ^= c3;
                    b4 ^= c4;
                }
                hit = ((tgt & 1) ? b0 : ~b0) & ((tgt & 2) ? b1 : ~b1) & ((tgt & 4) ? b2 : ~b2) &
                      ((tgt & 8) ? b3 : ~b3) & ((tgt & 16) ? b4 : ~b4) & lmask;
                // the count is read only for entries some candidate hits
                if (hit && (cov_ldcg(&d.cw[cov_ldcg(&d.ul_idx[c0 + (uint32_t)k])]) & 0xffffu) != 0) hit = 0;
            }
            const uint64_t eq = valid ? (~cov_spread(px ^ pu) & nm) : 0ull;
            for (int l = 0; l < nL; l++) {
                const uint32_t m = __ballot_sync(0xffffffffu, (hit >> l) & 1ull);
                if (lane == 0) LM[l * NG + (g ^ (l & (NG - 1)))] = m;
            }
            for (int j = 0; j < n; j++) {
                const uint32_t m = __ballot_sync(0xffffffffu, (eq >> (4 * j)) & 1ull);
                if (lane == 0) EJ[j * NG + (g ^ (j & (NG - 1)))] = m;
            }
        }
        cov_bar();
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int t = (int)threadIdx.x + u * NT;
            if (t < npair) {
                const int l = t / n, j = t - l * n;
                if ((S.Pmask[l] >> j) & 1) {
                    int sum = 0;
                    for (int g = 0; g < ng; g++)
                        sum += __popc(LM[l * NG + (g ^ (l & (NG - 1)))] & EJ[j * NG + (g ^ (j & (NG - 1)))]);
                    if (u == 0) acc0 += sum; else acc1 += sum;
                }
            }
        }
        cov_bar();
    }
    if (acc0) atomicAdd(&negp[threadIdx.x], acc0);
    if (acc1) atomicAdd(&negp[threadIdx.x + NT], acc1);
}

// candidate mask table for the bit-sliced list pass (nL <= 64)
__device__ void build_cmask(const CovSlot &d, Smem &S, int nL, uint64_t pu)
{
    for (int l = threadIdx.x; l < nL && l < L_SM; l += NT) {
        uint32_t P = 0;
        for (uint64_t m = cov_spread(S.Lpk[l] ^ pu); m; m &= m - 1) P |= 1u << ((__ffsll((long long)m) - 1) >> 2);
        S.Pmask[l] = (uint16_t)P;
    }
    const int nq = d.n * d.q;
    for (int t = threadIdx.x; t < nq; t += NT) {
        const int j = t / d.q, v = t - j * d.q;
        uint64_t m = 0;
        for (int l = 0; l < nL && l < 64; l++)
            if (cov_nib(S.Lpk[l], j) == v) m |= 1ull << l;
        S.cmask[t] = m;
    }
}

// Entering counts of every single-coordinate move of the candidate
// codewords (--wide, covsearch2e.c:720-733): for each current list entry x
// and each candidate l at distance exactly R+1 from it, negw[l][j][x_j]
// gains 1 at the R+1 positions j where they differ.  Up to 64 candidates
// held in shared memory find their hits by the bit-sliced count of equal
// positions over cmask; more are tested one by one.
__device__ __noinline__ void ul_pass_wide(const CovSlot &d, const Smem &S, int nL, bool sm, const uint32_t *Lp,
                             int32_t *negw, uint32_t first, uint32_t stride, uint32_t n0)
{
    const int n = d.n, q = d.q, R = d.R;
    const int tgt = n - (R + 1);
    const bool sliced = sm && nL <= 64 && d.wide_sliced;
    const uint64_t lmask = nL >= 64 ? ~0ull : ((1ull << nL) - 1);
    for (uint32_t e = first; e < n0; e += stride) {
        const uint64_t px = cov_ldcg(&d.ul_pk[e]);
        if (sliced) {
            uint64_t b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0;
            for (int j = 0; j < n; j++) {
                const uint64_t m = S.cmask[j * q + cov_nib(px, j)];
                uint64_t c1 = b0 & m; b0 ^= m;
                uint64_t c2 = b1 & c1; b1 ^= c1;
                uint64_t c3 = b2 & c2; b2 ^= c2;
                uint64_t c4 = b3 & c3; b3 ^= c3;
                b4 ^= c4;
            }
            uint64_t hit = ((tgt & 1) ? b0 : ~b0) & ((tgt & 2) ? b1 : ~b1) & ((tgt & 4) ? b2 : ~b2) &
                           ((tgt & 8) ? b3 : ~b3) & ((tgt & 16) ? b4 : ~b4) & lmask;
            if (!hit) continue;
            if ((cov_ldcg(&d.cw[cov_ldcg(&d.ul_idx[e])]) & 0xffffu) != 0) continue;   // stale entry
            for (; hit; hit &= hit - 1) {
                const int l = __ffsll((long long)hit) - 1;
                for (uint64_t m = cov_spread(px ^ S.Lpk[l]); m; m &= m - 1) {
                    const int j = (__ffsll((long long)m) - 1) >> 2;
                    atomicAdd(&negw[(l * n + j) * q + cov_nib(px, j)], 1);
                }
            }
            continue;
        }
        if ((cov_ldcg(&d.cw[cov_ldcg(&d.ul_idx[e])]) & 0xffffu) != 0) continue;
        for (int l = 0; l < nL; l++) {
            const uint64_t pk = sm ? S.Lpk[l] : cov_ldcg(&d.code[Lp[l]]);
            const uint64_t D = cov_spread(px ^ pk);
            if (__popcll(D) != R + 1) continue;
            for (uint64_t m = D; m; m &= m - 1) {
                const int j = (__ffsll((long long)m) - 1) >> 2;
                atomicAdd(&negw[(l * n + j) * q + cov_nib(px, j)], 1);
            }
        }
    }
}

// the list pass shared by the whole cluster: every CTA takes a slice of
// the list; the followers accumulate locally and add into the leader's counts
__device__ void op_neg(const CovSlot &d, const OpParams &P, Smem &S, Smem *LS, int rank, int csize)
{
    const int nL = P.nL, n = d.n;
    const uint32_t n0 = (uint32_t)P.uln;
    if (P.wide) {
        // every CTA adds its strided share of the list straight into g_negw
        if (rank != 0) {
            for (int l = threadIdx.x; l < nL; l += NT) S.Lpk[l] = LS->Lpk[l];
            for (int t = threadIdx.x; t < d.n * d.q; t += NT) S.cmask[t] = LS->cmask[t];
            cov_bar();
        }
        ul_pass_wide(d, S, nL, true, nullptr, d.g_negw, (uint32_t)rank * NT + threadIdx.x,
                     (uint32_t)(csize * NT), n0);
        return;
    }
    if (nL <= 64) {
        // contiguous slice of the list per CTA; counts go straight into the
        // leader's neg (one atomic per candidate and position per chunk)
        if (rank != 0) {
            for (int l = threadIdx.x; l < nL; l += NT) { S.Lpk[l] = LS->Lpk[l]; S.Pmask[l] = LS->Pmask[l]; }
            for (int t = threadIdx.x; t < d.n * d.q; t += NT) S.cmask[t] = LS->cmask[t];
            cov_bar();
        }
        const uint32_t per = (n0 + (uint32_t)csize - 1) / (uint32_t)csize;
        const uint32_t e0 = min(n0, (uint32_t)rank * per), e1 = min(n0, e0 + per);
        neg_chunks(d, S, P.pu, nL, e0, e1, LS->neg);
        return;
    }
    if (rank != 0) {
        for (int l = threadIdx.x; l < nL; l += NT) S.Lpk[l] = LS->Lpk[l];
        for (int t = threadIdx.x; t < d.n * d.q; t += NT) S.cmask[t] = LS->cmask[t];
        for (int x = threadIdx.x; x < nL * n; x += NT) S.neg[x] = 0;
        cov_bar();
    }
    ul_pass(d, P.pu, nL, S.Lpk, S.neg, (uint32_t)rank * NT + threadIdx.x, (uint32_t)(csize * NT), n0);
    if (rank != 0) {
        cov_bar();
        for (int x = threadIdx.x; x < nL * n; x += NT)
            if (S.neg[x]) atomicAdd(&LS->neg[x], S.neg[x]);
    }
}

// ----------------------------------------------------- leader routines -----
// pick_uncovered (covsearch2e.c:973-1016, opt_upick = opt_ucache = 0):
// 64 uniform probes, then the first zero cyclically after a random start.
// The probes are drawn up front and the RNG is advanced by exactly the
// number the reference consumes.
__device__ long long leader_pick(const CovSlot &d, Smem &S)
{
    const int tid = threadIdx.x;
    if (tid == 0) rs_ensure(S, 65);
    __syncwarp();
    cov_bar();
    if (tid < 64) {
        uint32_t w = (uint32_t)(rs_peek(S, tid) % (uint64_t)d.N);
        unsigned m = __ballot_sync(0xffffffffu, cnt_of(d, w) == 0);
        if ((tid & 31) == 0) S.hitmask[tid >> 5] = m;
    }
    cov_bar();
    int first = -1;
    if (S.hitmask[0]) first = __ffs(S.hitmask[0]) - 1;
    else if (S.hitmask[1]) first = 32 + __ffs(S.hitmask[1]) - 1;
    const int consumed = first >= 0 ? first + 1 : 65;
    long long result = -1;
    uint32_t start = 0;
    if (first >= 0) result = (long long)(rs_peek(S, first) % (uint64_t)d.N);
    else start = (uint32_t)(rs_peek(S, 64) % (uint64_t)d.N);
    cov_bar();
    if (tid == 0) S.rs_use += consumed;
    __syncwarp();
    if (first >= 0 || S.unc <= 0) return result;     // no zero anywhere: -1
    // Both searches below return the first zero after start.  The list is
    // scanned whole; the linear scan stops at the first zero, about q^n/unc
    // words on: it is the cheaper one while that distance is short.
    if (S.ul_valid && (unsigned long long)S.unc * 16384ull < (unsigned long long)d.N) {
        // every zero-count word is on the list: the first one after start is
        // the entry minimising (x - start) mod N
        // a thread reads the count only for an entry that would lower its
        // running minimum (a few per thread), not for every entry
        const int n0 = S.uln;
        unsigned best = 0xffffffffu;
        for (int e = tid; e < n0; e += NT) {
            uint32_t x = cov_ldcg(&d.ul_idx[e]);
            unsigned key = x >= start ? x - start : x + (d.N - start);
            if (key < best && (cov_ldcg(&d.cw[x]) & 0xffffu) == 0) best = key;
        }
        best = block_min_u32(S, best);
        if (best != 0xffffffffu) {
            // (start + best) may pass 2^32 when q^n > 2^31
            unsigned long long x = (unsigned long long)start + best;
            if (x >= d.N) x -= d.N;
            return (long long)x;
        }
        if (tid == 0) set_error(d, COV_EDRIFT);
        __syncwarp();
        return -1;
    }
    // chunked linear scan from start: PK consecutive counters per thread,
    // all loaded before any is tested
    constexpr int PK = 8;
    for (uint32_t off = 0; off < d.N; off += NT * PK) {
        unsigned best = 0xffffffffu;
        uint32_t c[PK];
#pragma unroll
        for (int k = 0; k < PK; k++) {
            const uint32_t o2 = off + (uint32_t)tid * PK + k;
            c[k] = 1;
            if (o2 < d.N) {
                unsigned long long x = (unsigned long long)start + o2;
                if (x >= d.N) x -= d.N;
                c[k] = cov_ldcg(&d.cw[x]) & 0xffffu;
            }
        }
#pragma unroll
        for (int k = PK - 1; k >= 0; k--)
            if (c[k] == 0) best = off + (uint32_t)tid * PK + (uint32_t)k;
        best = block_min_u32(S, best);
        if (best != 0xffffffffu) {
            unsigned long long x = (unsigned long long)start + best;
            if (x >= d.N) x -= d.N;
            return (long long)x;
        }
    }
    if (tid == 0) set_error(d, COV_EDRIFT);
    __syncwarp();
    return -1;
}

// drop list entries that are covered again (covsearch2e.c:305-320)
__device__ void leader_compact(const CovSlot &d, Smem &S)
{
    const int n0 = S.uln;
    int m = 0;
    for (int c0 = 0; c0 < n0; c0 += NT) {
        int e = c0 + threadIdx.x;
        int keep = 0;
        uint32_t x = 0; uint64_t pk = 0;
        if (e < n0) {
            x = cov_ldcg(&d.ul_idx[e]);
            pk = cov_ldcg(&d.ul_pk[e]);
            keep = (cov_ldcg(&d.cw[x]) & 0xffffu) == 0;
            if (!keep) atomicAnd(&d.ul_bit[x >> 5], ~(1u << (x & 31)));
        }
        int pos;
        int tot = block_excl_scan(S, keep, pos);
        if (keep) { cov_stcg(&d.ul_idx[m + pos], x); cov_stcg(&d.ul_pk[m + pos], pk); }
        m += tot;
        cov_bar();
    }
    if (threadIdx.x == 0) { d.st->ul_n = m; S.uln = m; }
    __syncwarp();
    cov_bar();
}

// Fisher-Yates resolved in parallel (shared-memory case, take <= PERM_CAP).
// Step s swaps positions s and j_s >= s.  Position x changes before step s
// only through earlier steps that target it, so with
//   prevT(t) = last step t' < t with j_t' = t          (position t's feeder)
//   W(t)     = value at position t when step t begins = W(prevT(t)) or t
// the value sampled at step s is W(prevS(s)) when some earlier step
// targeted j_s (prevS(s) = the last one), else j_s itself.  Steps are
// bucketed by target (counting sort), each bucket sorted by step, and W
// follows prevT chains by pointer jumping.  j_s arrives in dval[s]; the
// result is written to perm[0..take).  ncand entries of fy_a/fy_b are used.
__device__ void fy_parallel(Smem &S, int take, int ncand)
{
    const int tid = threadIdx.x;
    int32_t *cnt = S.fy_a;        // per position: number of steps targeting it, then bucket start
    int32_t *bkt = S.fy_b;        // bucketed step ids
    uint32_t *perm = S.perm;
    const int32_t *jv = S.dval;
    for (int x = tid; x < ncand; x += NT) cnt[x] = 0;
    cov_bar();
    for (int s = tid; s < take; s += NT) atomicAdd(&cnt[jv[s]], 1);
    cov_bar();
    // exclusive prefix over positions, NT-chunked
    {
        const int CH = (ncand + NT - 1) / NT;
        const int lo = min(ncand, tid * CH), hi = min(ncand, lo + CH);
        int loc = 0;
        for (int x = lo; x < hi; x++) loc += cnt[x];
        int tot;
        int pre = block_scan_int(S, loc, 0, [](int a, int b) { return a + b; }, tot);
        for (int x = lo; x < hi; x++) { int c = cnt[x]; cnt[x] = pre; pre += c; }
    }
    cov_bar();
    // place steps; cnt[x] becomes the end of bucket x
    for (int s = tid; s < take; s += NT) {
        const int slot = atomicAdd(&cnt[jv[s]], 1);
        bkt[slot] = s;
    }
    cov_bar();
    // sort each bucket by step (buckets are tiny); bucket x = [start, end)
    for (int x = tid; x < ncand; x += NT) {
        const int end = cnt[x];
        int start = end;
        // start of bucket x = end of bucket x-1 (cnt is an end pointer now)
        start = x ? cnt[x - 1] : 0;
        for (int a = start + 1; a < end; a++) {
            int v = bkt[a], b = a - 1;
            while (b >= start && bkt[b] > v) { bkt[b + 1] = bkt[b]; b--; }
            bkt[b + 1] = v;
        }
    }
    cov_bar();
    // one thread per bucket (= position x): prevS for its steps and, for
    // x < take, prevT(x) = the last step < x targeting x
    int32_t *prevS = reinterpret_cast<int32_t *>(perm);   // perm[0..take) reused
    for (int x = tid; x < ncand; x += NT) {
        const int start = x ? cnt[x - 1] : 0, end = cnt[x];
        int pt = -1;
        for (int a = start; a < end; a++) {
            const int st = bkt[a];
            prevS[st] = a > start ? bkt[a - 1] : -1;
            if (st < x) pt = st;
        }
        if (x < take) S.fy_c[x] = pt;
    }
    cov_bar();
    // W by pointer jumping: w[t] is a step index until its chain is resolved,
    // then -(value + 1).  Chains strictly decrease, so they end.
    int32_t *w = S.fy_a;
    for (int t = tid; t < take; t += NT) {
        const int pt = S.fy_c[t];
        w[t] = pt < 0 ? -(t + 1) : pt;
    }
    cov_bar();
    for (int round = 0; round < 16; round++) {
        int changed = 0;
        for (int t = tid; t < take; t += NT) {
            const int a = w[t];
            if (a >= 0) { w[t] = w[a]; changed = 1; }
        }
        changed = cov_bar_or(changed);
        if (!changed) break;
    }
    // perm[s] = W(prevS(s)) or j_s
    for (int s = tid; s < take; s += NT) {
        const int ps = prevS[s];
        perm[s] = (uint32_t)(ps >= 0 ? -(w[ps] + 1) : jv[s]);
    }
    cov_bar();
}

__device__ void zero_acc(Smem &S)
{
    if (threadIdx.x == 0) { S.acc.dunc = 0; S.acc.accT = 0; }
    __syncwarp();
    if (threadIdx.x < COV_MAXN) S.acc.accH[threadIdx.x] = 0;
}

__device__ void issue_move(const CovSlot &d, Smem &S, int k, uint64_t pk, int p, int v, long long dd);
__device__ bool method_pick(const CovSlot &d, Smem &S, uint32_t *Lp);
__device__ void write_trace(const CovSlot &d, Smem &S);
__device__ void copy_best(const CovSlot &d);

// Plan one iteration up to the point where the entering-side counts are
// needed.  Returns with S.opp set.
__device__ void leader_plan(const CovSlot &d, Smem &S, int csize)
{
    const int tid = threadIdx.x;
    const int n = d.n, R = d.R, M = d.M;
    if (tid == 0) {
        const int u = cov_ldcg(&d.st->ul_n);
        if (S.ul_valid && u > d.ul_cap) S.ul_valid = 0;
        S.uln = min(u, d.ul_cap);
        int stop = S.status != 0 || S.unc <= 0 || S.moves_left <= 0 ||
                   (S.target >= 0 && S.best_unc <= S.target);
        const bool late = (unsigned long long)cov_clock() > S.t_deadline;
        if (!stop && late) S.status = COV_ETIMEOUT;
        stop = stop || late;
        S.ibc[0] = stop;
        S.ibc[1] = !stop && !S.ul_valid && S.unc <= d.ul_cap / 2;
    }
    __syncwarp();
    cov_bar();
    if (S.ibc[0]) {
        if (tid == 0) { S.opp.op = OP_STOP; S.phase = PH_STOPPED; }
        __syncwarp();
        return;
    }
    if (S.ibc[1]) {
        if (tid == 0) {
            d.st->ul_n = 0;
            S.opp.op = OP_REBUILD_UL;
            S.phase = PH_REBUILD_DONE;
        }
        __syncwarp();
        return;
    }
    long long t0 = cov_clock();
    if (S.ul_valid && (long long)S.uln > 2 * S.unc + 64) leader_compact(d, S);
    if (tid == 0) {
        long long t1 = cov_clock();
        S.prof[6] += t1 - t0;
        t0 = t1;
        S.it++;
        S.moves_left--;
        memset(&S.rec, 0, sizeof(S.rec));
        S.rec.it = S.it;
    }
    __syncwarp();
    cov_bar();
    long long uw = leader_pick(d, S);
    if (tid == 0) {
        long long t1 = cov_clock();
        S.prof[0] += t1 - t0;
        t0 = t1;
        S.uw = uw;
        if (uw < 0) S.status = COV_EDRIFT;
        S.pu = uw >= 0 ? pk_of_idx(d, (uint32_t)uw) : 0;
        S.rec.u = uw;
    }
    __syncwarp();
    cov_bar();
    if (S.status) { if (tid == 0) { S.opp.op = OP_STOP; S.phase = PH_STOPPED; } return; }
    const uint64_t pu = S.pu;

    // distances to all codewords and the target distance (covsearch2e.c:1342-1351)
    const bool csm = M <= CODE_SM;
    unsigned dm = 0xffffffffu;
    // (with --fix0 codeword 0 is not a candidate, covsearch2e.c:1343)
    for (int i = tid; i < M; i += NT) {
        if (i < d.fix0) { if (csm) S.dist8[i] = 0xff; continue; }
        int dd = cov_dist(leader_code(d, S, i), pu);
        if (csm) S.dist8[i] = (uint8_t)dd;
        dm = min(dm, (unsigned)dd);
    }
    dm = block_min_u32(S, dm);
    if (tid == 0) { long long t1 = cov_clock(); S.prof[10] += t1 - t0; }
    __syncwarp();
    const int dtar = ((int)dm <= R + 1) ? R + 1 : (int)dm;
    // ordered list of codewords at distance dtar (covsearch2e.c:1359-1376):
    // always in global memory, the first L_SM also in shared memory with
    // their packed codes and one-hot masks
    int nL = 0;
    for (int c0 = 0; c0 < M; c0 += NT) {
        int i = c0 + tid;
        uint64_t pk = 0;
        int f = 0;
        if (i < M && i >= d.fix0) {
            pk = leader_code(d, S, i);
            f = (csm ? (int)S.dist8[i] : cov_dist(pk, pu)) == dtar;
        }
        int pos;
        int tot = block_excl_scan(S, f, pos);
        if (f) {
            const int at = nL + pos;
            d.g_list[at] = (uint32_t)i;
            if (at < L_SM) {
                S.L[at] = (uint32_t)i;
                S.Lpk[at] = pk;
            }
        }
        nL += tot;
    }
    int Lsm = nL <= L_SM;
    uint32_t *Lp = Lsm ? S.L : d.g_list;
    // --wide (covsearch2e.c:1353-1376): while the list is valid and
    // U_n n < (R+1) S', the candidates are all n(q-1) moves of each
    // codeword at dtar (p outer, v inner, v != c_p); else the dtar moves
    // towards u
    const bool wide_now = d.wide && S.ul_valid &&
        (long long)S.uln * n < (long long)(R + 1) * (long long)d.nsub * (long long)d.ppow[R];
    const int cpw = wide_now ? n * (d.q - 1) : dtar;
    const int ncand = nL * cpw;
    if (ncand == 0) {     // impossible for an uncovered target word
        if (tid == 0) { S.status = COV_EDRIFT; S.opp.op = OP_STOP; S.phase = PH_STOPPED; }
        __syncwarp();
        return;
    }
    const int take = min(ncand, d.cand);
    const int psm = ncand <= PERM_CAP;
    uint32_t *perm = psm ? S.perm : d.g_perm;
    int32_t *dval = psm ? S.dval : d.g_dval;
    for (int c = tid; c < ncand; c += NT) perm[c] = (uint32_t)c;
    // Fisher-Yates sample of `take` (covsearch2e.c:1383-1389): the draws are
    // generated in order by one thread, reduced in parallel, applied in order.
    for (int s0 = 0; s0 < take; s0 += RB) {
        const int cnt = min(RB, take - s0);
        cov_bar();
        if (tid == 0) rs_ensure(S, cnt);
        __syncwarp();
        cov_bar();
        for (int t = tid; t < cnt; t += NT) {
            int s = s0 + t;
            dval[s] = s + (int32_t)fastmod(S, rs_peek(S, t), (uint64_t)(ncand - s));
        }
        cov_bar();
        if (tid == 0) S.rs_use += cnt;
        __syncwarp();
    }
    cov_bar();
    // the sample's permutation: in parallel in shared memory; the oversized
    // case is swapped in order by one thread while the others work on the
    // entering side (apply_swaps), which does not need it
    int pending = 1;
    if (psm) {
        // perm[c] = c was set above for c < ncand; fy_parallel rewrites
        // perm[0..take) directly from the draws
        fy_parallel(S, take, ncand);
        pending = 0;
        if (take < ncand && tid == 0) {
            int c = 0;
            for (int s2 = 0; s2 < take; s2++) {
                int l = (int)(perm[s2] / (uint32_t)cpw), dup = 0;
                for (int t2 = 0; t2 < s2; t2++) if ((int)(perm[t2] / (uint32_t)cpw) == l) { dup = 1; break; }
                c += !dup;
            }
            S.ibc[2] = c;
        }
        cov_bar();
    }
    if (tid == 0) {
        S.swaps_pending = pending;
        S.nL = nL; S.dtar = dtar; S.ncand = ncand; S.take = take;
        S.cpw = cpw; S.wide_now = wide_now;
        S.rec.ncand = ncand; S.rec.ncw = (!pending && take < ncand) ? S.ibc[2] : nL;
        long long t1 = cov_clock();
        S.prof[1] += t1 - t0;
        t0 = t1;
    }
    __syncwarp();
    // --noise / --sa (covsearch2e.c:1408-1448): a move drawn from the sample
    // before any evaluation.  A noisy move is committed as it is; an
    // annealing proposal is evaluated alone (its codeword is the whole list)
    if (d.sa || d.noise) {
        cov_bar();
        if (tid == 0) S.ibc[0] = method_pick(d, S, Lp) ? 1 : 0;
        __syncwarp();
        cov_bar();
        if (S.noisy) return;                   // OP_MOVE issued
        if (S.ibc[0]) {                         // --sa: the proposal's codeword alone
            nL = 1;
            Lsm = 1;
            Lp = S.L;
        }
    }
    // entering side
    const int nsm = nL <= L_SM;
    int32_t *negp = nsm ? S.neg : d.g_neg;
    for (int x = tid; x < nL * n; x += NT) negp[x] = 0;
    zero_acc(S);
    cov_bar();
    if (tid == 0) {
        // per-move workload counters: candidate codewords, list length, moves
        S.prof[20] += (unsigned long long)nL;
        S.prof[21] += S.ul_valid ? (unsigned long long)S.uln : 0ull;
        S.prof[22] += 1;
    }
    if (wide_now) {
        // one list pass gives the entering count of every (l, j, v)
        int32_t *negw = d.g_negw;
        for (int x = tid; x < nL * n * d.q; x += NT) cov_stcg(&negw[x], 0);
        if (Lsm && nL <= 64) build_cmask(d, S, nL, pu);
        cov_bar();
        const long long pairs = (long long)S.uln * nL;
        if (csize > 1 && Lsm && pairs >= d.neg_cluster_pairs) {
            if (tid == 0) {
                OpParams &o = S.opp;
                o.op = OP_NEG; o.nL = nL; o.dtar = dtar; o.pu = pu; o.uln = S.uln;
                o.L_sm = 1; o.neg_sm = 1; o.ul_valid = 1; o.wide = 1;
                S.phase = PH_SELECT;
                S.prof[2] += cov_clock() - t0;
                S.ul_pairs += pairs;
            }
            __syncwarp();
            return;
        }
        ul_pass_wide(d, S, nL, Lsm, Lp, negw, tid, NT, (uint32_t)S.uln);
        cov_bar();
        if (tid == 0) {
            S.phase = PH_SELECT;
            S.prof[2] += cov_clock() - t0;
            S.ul_pairs += pairs;
        }
        __syncwarp();
        S.opp.op = -1;
        return;
    }
    // The list and the walk give the same counts (covsearch2e.c:720-753);
    // the reference picks the list while U_n n < (R+1) S' (:1466-1467).  Here
    // the list costs per entry whatever the number of candidates (one mask
    // test for up to 64), the walk per candidate: list while
    // U_n * list_cost < ncw (R+1) S'.
    const bool use_list = S.ul_valid &&
        (long long)S.uln * d.list_cost < (long long)nL * (R + 1) * (long long)d.nsub * (long long)d.ppow[R];
    if (!use_list) {
        if (tid == 0) {
            apply_swaps(d, S);
            OpParams &o = S.opp;
            o.op = OP_NEGWALK; o.nL = nL; o.dtar = dtar; o.pu = pu;
            o.L_sm = Lsm; o.neg_sm = nsm; o.ul_valid = 0;
            S.phase = PH_SELECT;
        }
        __syncwarp();
        return;
    }
    if (Lsm) build_cmask(d, S, nL, pu);
    cov_bar();
    const long long pairs = (long long)S.uln * nL;
    long long tp0 = 0;
    if (tid == 0) tp0 = cov_clock();
    __syncwarp();
    if (csize > 1 && Lsm && pairs >= d.neg_cluster_pairs) {
        if (tid == 0) {
            OpParams &o = S.opp;
            o.op = OP_NEG; o.nL = nL; o.dtar = dtar; o.pu = pu; o.uln = S.uln;
            o.L_sm = 1; o.neg_sm = 1; o.ul_valid = 1; o.wide = 0;
            S.phase = PH_SELECT;
            S.prof[2] += cov_clock() - t0;
            S.ul_pairs += pairs;
        }
        __syncwarp();
        return;
    }
    if (Lsm && nL <= 64) {
        neg_chunks(d, S, pu, nL, 0, (uint32_t)S.uln, negp);
        if (tid == 0) S.prof[13] += cov_clock() - tp0;
        __syncwarp();
    } else if (Lsm) {
        ul_pass(d, pu, nL, S.Lpk, negp, tid, NT, (uint32_t)S.uln);
        cov_bar();
    } else {
        if (tid == 0) apply_swaps(d, S);
        __syncwarp();
        // oversized candidate list: codes from global memory, nibble test
        const int n0 = S.uln;
        const uint64_t nm = nibmask(n);
        for (int e = tid; e < n0; e += NT) {
            uint32_t x = cov_ldcg(&d.ul_idx[e]);
            if ((cov_ldcg(&d.cw[x]) & 0xffffu) != 0) continue;
            uint64_t px = cov_ldcg(&d.ul_pk[e]);
            uint64_t eq = ~cov_spread(px ^ pu) & nm;
            for (int l = 0; l < nL; l++) {
                uint64_t pk = cov_ldcg(&d.code[Lp[l]]);
                uint64_t D = cov_spread(px ^ pk);
                if (__popcll(D) != R + 1) continue;
                uint64_t m = D & eq;
                while (m) {
                    int j = (__ffsll((long long)m) - 1) >> 2;
                    atomicAdd(&negp[l * n + j], 1);
                    m &= m - 1;
                }
            }
        }
    }
    cov_bar();
    if (tid == 0) {
        S.phase = PH_SELECT;
        S.prof[2] += cov_clock() - t0;
        S.ul_pairs += (long long)S.uln * nL;
    }
    __syncwarp();
    S.opp.op = -1;   // no op yet: select follows
}

// Candidate r of codeword pk: position and value (covsearch2e.c:1359-1376).
// Plain: the r-th position where pk differs from u, moved to u's digit.
// Wide: r = p (q-1) + the rank of v among the values other than c_p.
__device__ __forceinline__ void cand_pv(const CovSlot &d, bool wide, int r, uint64_t pk, uint64_t pu,
                                        int &p, int &v)
{
    if (wide) {
        const int qm1 = d.q - 1;
        p = r / qm1;
        const int vv = r - p * qm1;
        v = vv + (vv >= cov_nib(pk, p));
    } else {
        p = nth_set_pos(cov_spread(pk ^ pu), r);
        v = cov_nib(pu, p);
    }
}

// entering count of candidate l's move (p, v)
__device__ __forceinline__ int cand_neg(const CovSlot &d, bool wide, const int32_t *negp, int l, int p, int v)
{
    return wide ? cov_ldcg(&d.g_negw[(l * d.n + p) * d.q + v]) : negp[l * d.n + p];
}

// OP_MOVE of codeword k (packed pk) at position p to value v, evaluated
// delta dd
__device__ void issue_move(const CovSlot &d, Smem &S, int k, uint64_t pk, int p, int v, long long dd)
{
    S.chosen_delta = dd;
    OpParams &o = S.opp;
    o.op = OP_MOVE;
    o.mi = k; o.mp = p; o.mv = v; o.sgn = 0;
    o.ul_valid = S.ul_valid;
    o.pc = pk;
    o.base = widx_pk(d, pk);
    const int oldv = cov_nib(pk, p);
    o.dv = (uint32_t)((long long)(v - oldv) * (long long)d.pw[p]);
    o.pcn = cov_setnib(pk, p, v);
    o.basen = o.base + o.dv;
    S.ibc[3] = oldv;
    S.rec.i = k; S.rec.p = p; S.rec.v = v; S.rec.delta = dd;
}

// --noise and --sa, after the candidate sample (one thread).  --noise
// (covsearch2e.c:1443-1448): with probability noise/1000 a sampled move is
// committed unevaluated; the move is issued and S.noisy set.  --sa
// (:1408-1414): one sampled move is proposed; its codeword becomes the whole
// candidate list (L[0]) so that the entering side counts only its moves, and
// true is returned.  The draws are the reference's, in its order.
__device__ bool method_pick(const CovSlot &d, Smem &S, uint32_t *Lp)
{
    S.noisy = 0;
    int s = -1;
    if (d.sa) s = (int)fastmod(S, rs_take(S), (uint64_t)S.take);
    else if ((int)fastmod(S, rs_take(S), 1000ull) < d.noise) {
        S.noisy = 1;
        s = (int)fastmod(S, rs_take(S), (uint64_t)S.take);
    }
    if (s < 0) return false;
    apply_swaps(d, S);                          // the sample's order
    const int psm = S.ncand <= PERM_CAP;
    const uint32_t c = (psm ? S.perm : d.g_perm)[s];
    const int l = (int)(c / (uint32_t)S.cpw), r = (int)(c - (uint32_t)l * S.cpw);
    const int k = (int)Lp[l];
    const uint64_t pk = cov_ldcg(&d.code[k]);
    int p, v;
    cand_pv(d, S.wide_now, r, pk, S.pu, p, v);
    if (S.noisy) {
        // the entering side is skipped, and with it the accumulators' reset
        S.acc.dunc = 0;
        S.acc.accT = 0;
        for (int j = 0; j < COV_MAXN; j++) S.acc.accH[j] = 0;
        issue_move(d, S, k, pk, p, v, 0);
        S.phase = PH_FINISH_MOVE;
        return false;
    }
    S.L[0] = (uint32_t)k;
    S.Lpk[0] = pk;
    S.nL = 1;
    S.sa_p = p;
    S.sa_v = v;
    S.rec.ncw = 1;
    return true;
}

// --sa (covsearch2e.c:1415-1420): the proposal's exact delta and the
// Metropolis test; an accepted move is issued (one thread)
__device__ void sa_decide(const CovSlot &d, Smem &S)
{
    const int k = (int)S.L[0], p = S.sa_p, v = S.sa_v;
    const uint64_t pk = S.Lpk[0];
    const int32_t *Pk = d.P + (size_t)k * (d.n + 1);
    const long long dd = (cov_ldcg(&Pk[0]) - cov_ldcg(&Pk[1 + p])) - cand_neg(d, S.wide_now, S.neg, 0, p, v);
    int accept = dd <= 0;
    if (!accept) {
        const double pr = exp(-(double)dd / S.sa_T);
        accept = (double)(rs_take(S) >> 11) * 0x1.0p-53 < pr;
    }
    S.sa_accept = accept;
    S.rec.i = k; S.rec.p = p; S.rec.v = v; S.rec.delta = dd;
    if (accept) issue_move(d, S, k, pk, p, v, dd);
    else S.opp.op = -1;
    S.phase = PH_SA_END;
}

// --sa, after the proposal (covsearch2e.c:1421-1441): the accepted move's
// bookkeeping (no tabu), the cooling schedule and the stall reheat
__device__ void leader_sa_end(const CovSlot &d, Smem &S)
{
    const int tid = threadIdx.x;
    const int n = d.n;
    if (tid == 0) {
        S.improved = 0;
        S.rec.kicked = S.sa_accept ? 0 : 2;    // bit 1: rejected
        if (S.sa_accept) {
            const long long dunc = (long long)S.acc.dunc;
            S.unc += dunc;
            if (dunc != S.chosen_delta) S.status = COV_EDRIFT;
            const OpParams &o = S.opp;
            leader_set_code(d, S, o.mi, o.pcn);
            int32_t *Pk = d.P + (size_t)o.mi * (n + 1);
            cov_stcg(&Pk[0], cov_ldcg(&Pk[0]) + S.acc.accT);
            for (int j = 0; j < n; j++) cov_stcg(&Pk[1 + j], cov_ldcg(&Pk[1 + j]) + S.acc.accH[j]);
            S.improved = S.unc < S.best_unc;
            if (S.improved) { S.best_unc = S.unc; S.since_improve = 0; }
        }
        S.rec.unc = S.unc;
        S.sa_T *= d.sa_cool;
        if (S.sa_T < d.sa_tmin) S.sa_T = d.sa_t0;            // reheat
        if (++S.since_improve > d.stall) {
            S.sa_T = d.sa_t0;
            S.since_improve = 0;
            S.nkicks++;
            S.rec.kicked |= 1;                                // bit 0: the stall reheat
        }
    }
    __syncwarp();
    cov_bar();
    if (S.improved) copy_best(d);
    cov_bar();
    if (tid == 0) {
        S.rec.unc_end = S.unc;
        S.rec.best = S.best_unc;
        write_trace(d, S);
        S.phase = PH_PLAN;
    }
    __syncwarp();
    cov_bar();
}

// Deltas of the sampled candidates and the tabu/aspiration/reservoir
// selection of covsearch2e.c:1503-1518; emits OP_MOVE.
__device__ void leader_select(const CovSlot &d, Smem &S)
{
    const int tid = threadIdx.x;
    const int n = d.n, q = d.q;
    const int nL = S.nL, cpw = S.cpw, ncand = S.ncand, take = S.take;
    const bool wide = S.wide_now;
    const uint64_t pu = S.pu;
    const int psm = ncand <= PERM_CAP, Lsm = nL <= L_SM;
    uint32_t *perm = psm ? S.perm : d.g_perm;
    int32_t *dval = psm ? S.dval : d.g_dval;
    uint32_t *Lp = Lsm ? S.L : d.g_list;
    int32_t *negp = Lsm ? S.neg : d.g_neg;
    const long long t0 = cov_clock();
    if (tid == 0) apply_swaps(d, S);
    __syncwarp();
    cov_bar();
    if (d.sa) {
        if (tid == 0) { sa_decide(d, S); S.prof[3] += cov_clock() - t0; }
        __syncwarp();
        return;
    }
    // deltas and tabu flags in parallel (shared-memory case); the rare
    // oversized case recomputes them inside the serial scan below
    if (psm) {
        for (int s = tid; s < take; s += NT) {
            uint32_t c = perm[s];
            int l = (int)(c / (uint32_t)cpw), r = (int)(c - (uint32_t)l * cpw);
            int k = (int)Lp[l];
            uint64_t pk = Lsm ? S.Lpk[l] : cov_ldcg(&d.code[k]);
            int p, v;
            cand_pv(d, wide, r, pk, pu, p, v);
            const int32_t *Pk = d.P + (size_t)k * (n + 1);
            dval[s] = (cov_ldcg(&Pk[0]) - cov_ldcg(&Pk[1 + p])) - cand_neg(d, wide, negp, l, p, v);
            S.tflag[s] = (uint8_t)((long long)cov_ldcg(&d.tabu[((size_t)k * n + p) * q + v]) > S.it);
        }
    }
    cov_bar();
    // Selection (covsearch2e.c:1503-1518) in parallel.  Scanning s in order
    // with eligible keys d_s, a "reset" is an eligible s with d_s below the
    // running minimum and an "event" one equal to it; each event draws once
    // and, with nties = its rank in the current minimum's run (the reset
    // counting 1), replaces the choice when draw % nties == 0.  Only events
    // at the final minimum V can win: the last of them whose draw hits, else
    // the first position holding V.  With nothing eligible one draw picks a
    // random candidate.
    int bs_par = -2, consumed = 0;
    if (psm) {
        const long long unc = S.unc, best = S.best_unc;
        const int CH = (take + NT - 1) / NT;
        const int s_lo = min(take, tid * CH), s_hi = min(take, s_lo + CH);
        const int INF = 0x7fffffff;
        auto keyof = [&](int s2) -> int {
            const int dd = dval[s2];
            return (S.tflag[s2] && unc + dd >= best) ? INF : dd;
        };
        int cmin = INF;
        for (int s2 = s_lo; s2 < s_hi; s2++) cmin = min(cmin, keyof(s2));
        int V;
        const int pmin = block_scan_int(S, cmin, INF, [](int a2, int b2) { return min(a2, b2); }, V);
        // events per chunk and the event count at the chunk's last reset
        int m = pmin, nev = 0, ev_reset = -1;
        for (int s2 = s_lo; s2 < s_hi; s2++) {
            const int k2 = keyof(s2);
            if (k2 == INF) continue;
            if (k2 < m) { m = k2; ev_reset = nev; }
            else if (k2 == m) nev++;
        }
        int E;
        const int evbase = block_scan_int(S, nev, 0, [](int a2, int b2) { return a2 + b2; }, E);
        int dummy;
        const int in_reset = block_scan_int(S, ev_reset >= 0 ? evbase + ev_reset : -1, -1,
                                            [](int a2, int b2) { return b2 != -1 ? b2 : a2; }, dummy);
        if (V != INF && E <= RS / 2) {
            if (tid == 0) rs_ensure(S, E);
            __syncwarp();
            cov_bar();
            // first occurrence of V and the last winning event at V
            int firstV = INF, win = -1;
            m = pmin;
            int cur_reset = in_reset, g = evbase;
            for (int s2 = s_lo; s2 < s_hi; s2++) {
                const int k2 = keyof(s2);
                if (k2 == INF) continue;
                if (k2 < m) {
                    m = k2;
                    cur_reset = g;
                    if (k2 == V) firstV = min(firstV, s2);
                } else if (k2 == m) {
                    const int nties = 1 + (g + 1) - cur_reset;
                    if (k2 == V && fastmod(S, rs_peek(S, g), (uint64_t)nties) == 0) win = s2;
                    g++;
                }
            }
            int fv, wv;
            block_scan_int(S, firstV, INF, [](int a2, int b2) { return min(a2, b2); }, fv);
            block_scan_int(S, win, -1, [](int a2, int b2) { return max(a2, b2); }, wv);
            bs_par = wv >= 0 ? wv : fv;
            consumed = E;
        } else if (V == INF) {
            if (tid == 0) { rs_ensure(S, 1); }
            __syncwarp();
            cov_bar();
            bs_par = (int)fastmod(S, rs_peek(S, 0), (uint64_t)take);
            consumed = 1;
        }
    }
    if (tid == 0) {
        long long ts1 = cov_clock();
        S.prof[8] += ts1 - t0;
        int bs = -1;
        if (bs_par >= 0) {
            bs = bs_par;
            S.rs_use += consumed;
        } else {
            long long bestd = 1LL << 60;
            int nties = 0;
            for (int s = 0; s < take; s++) {
                long long dd;
                int tb;
                if (psm) { dd = dval[s]; tb = S.tflag[s]; }
                else {
                    uint32_t c = perm[s];
                    int l = (int)(c / (uint32_t)cpw), rr = (int)(c - (uint32_t)l * cpw);
                    int k = (int)Lp[l];
                    uint64_t pk = cov_ldcg(&d.code[k]);
                    int p, v;
                    cand_pv(d, wide, rr, pk, pu, p, v);
                    const int32_t *Pk = d.P + (size_t)k * (n + 1);
                    dd = (cov_ldcg(&Pk[0]) - cov_ldcg(&Pk[1 + p])) - cand_neg(d, wide, negp, l, p, v);
                    tb = (long long)cov_ldcg(&d.tabu[((size_t)k * n + p) * q + v]) > S.it;
                }
                if (tb && S.unc + dd >= S.best_unc) continue;
                if (dd < bestd) { bestd = dd; bs = s; nties = 1; }
                else if (dd == bestd) {
                    nties++;
                    if (fastmod(S, rs_take(S), (uint64_t)nties) == 0) bs = s;
                }
            }
            if (bs < 0) bs = (int)fastmod(S, rs_take(S), (uint64_t)take);
        }
        long long ts2 = cov_clock();
        S.prof[9] += ts2 - ts1;
        uint32_t c = perm[bs];
        int l = (int)(c / (uint32_t)cpw), rr = (int)(c - (uint32_t)l * cpw);
        int k = (int)Lp[l];
        uint64_t pk = cov_ldcg(&d.code[k]);
        int p, v;
        cand_pv(d, wide, rr, pk, pu, p, v);
        const int32_t *Pk = d.P + (size_t)k * (n + 1);
        long long dd = (cov_ldcg(&Pk[0]) - cov_ldcg(&Pk[1 + p])) - cand_neg(d, wide, negp, l, p, v);
        issue_move(d, S, k, pk, p, v, dd);
        S.phase = PH_FINISH_MOVE;
        S.prof[3] += cov_clock() - t0;
    }
    __syncwarp();
}

__device__ void write_trace(const CovSlot &d, Smem &S)
{
    if (d.trace && S.trace_n < d.trace_cap)
        reinterpret_cast<cov_move_rec *>(d.trace)[S.trace_n] = S.rec;
    if (d.trace) S.trace_n++;
}

__device__ void copy_best(const CovSlot &d)
{
    for (int i = threadIdx.x; i < d.M; i += NT) cov_stcg(&d.best[i], cov_ldcg(&d.code[i]));
}

// after OP_MOVE: covsearch2e.c:1525-1553
__device__ void leader_finish_move(const CovSlot &d, Smem &S)
{
    const int tid = threadIdx.x;
    const int n = d.n, q = d.q;
    const long long t0 = cov_clock();
    if (tid == 0) {
        long long dunc = (long long)S.acc.dunc;
        S.unc += dunc;
        if (S.noisy) S.rec.delta = dunc;        // --noise: the move was not evaluated
        else if (dunc != S.chosen_delta) S.status = COV_EDRIFT;
        const OpParams &o = S.opp;
        leader_set_code(d, S, o.mi, o.pcn);
        int32_t *Pk = d.P + (size_t)o.mi * (n + 1);
        cov_stcg(&Pk[0], cov_ldcg(&Pk[0]) + S.acc.accT);
        for (int j = 0; j < n; j++) cov_stcg(&Pk[1 + j], cov_ldcg(&Pk[1 + j]) + S.acc.accH[j]);
        const int oldv = S.ibc[3];
        uint64_t r4 = rs_take(S) % 4ull;
        cov_stcg(&d.tabu[((size_t)o.mi * n + o.mp) * q + oldv], (int32_t)(S.it + d.tenure + (long long)r4));
        S.rec.unc = S.unc;
        S.improved = S.unc < S.best_unc;
        S.dokick = 0;
        if (S.improved) { S.best_unc = S.unc; S.since_improve = 0; }
        else if (++S.since_improve > d.stall) S.dokick = 1;
    }
    __syncwarp();
    cov_bar();
    if (S.improved) copy_best(d);
    cov_bar();
    if (tid == 0) {
        if (S.dokick) { S.kick_t = 0; S.phase = PH_KICK_START; }
        else {
            S.rec.unc_end = S.unc; S.rec.best = S.best_unc;
            write_trace(d, S);
            S.phase = PH_PLAN;
        }
        S.prof[5] += cov_clock() - t0;
    }
    __syncwarp();
    cov_bar();
}

// one leader step: consume the result of the previous op, do the serial
// work, and leave the next op in S.opp
__device__ void leader_step(const CovSlot &d, Smem &S, int csize)
{
    const int tid = threadIdx.x;
    for (int guard = 0; guard < 64; guard++) {
        cov_bar();
        const int ph = S.phase;
        cov_bar();
        if (ph == PH_STOPPED) { if (tid == 0) S.opp.op = OP_STOP; return; }
        if (ph == PH_PLAN) {
            if (S.mode == MODE_GREEDY) { if (tid == 0) S.phase = PH_GREEDY; continue; }
            leader_plan(d, S, csize);
            cov_bar();
            if (S.phase == PH_SELECT && S.opp.op == -1) {
                leader_select(d, S);
                cov_bar();
                if (S.phase == PH_SA_END && S.opp.op == -1) continue;   // rejected proposal
            }
            return;
        }
        if (ph == PH_SELECT) {
            leader_select(d, S);
            cov_bar();
            if (S.phase == PH_SA_END && S.opp.op == -1) continue;       // rejected proposal
            return;
        }
        if (ph == PH_FINISH_MOVE) { leader_finish_move(d, S); continue; }
        if (ph == PH_SA_END) {
            // a finished --sa iteration: a rejected proposal issues no op, so
            // one step can run many iterations; each uses one move of the
            // launch's budget, which bounds the loop
            leader_sa_end(d, S);
            guard = 0;
            continue;
        }
        if (ph == PH_REBUILD_DONE) {
            if (tid == 0) {
                int cnt = cov_ldcg(&d.st->ul_n);
                S.ul_valid = cnt <= d.ul_cap;
                S.uln = min(cnt, d.ul_cap);
                S.phase = PH_PLAN;
            }
            __syncwarp();
            continue;
        }
        if (ph == PH_KICK_START) {
            if (tid == 0) {
                if (S.kick_t >= d.kick) {
                    S.opp.op = OP_ZERO_TABU;
                    S.phase = PH_KICK_DONE;
                } else {
                    const int cnt = cov_ldcg(&d.st->ul_n);
                    if (S.ul_valid && cnt > d.ul_cap) S.ul_valid = 0;
                    S.uln = min(cnt, d.ul_cap);
                    int i = d.fix0 + (int)fastmod(S, rs_take(S), (uint64_t)(d.M - d.fix0));
                    uint64_t pk = leader_code(d, S, i);
                    OpParams &o = S.opp;
                    o.op = OP_BALL; o.sgn = -1; o.mi = i; o.pc = pk; o.base = widx_pk(d, pk);
                    o.ul_valid = S.ul_valid;
                    S.acc.dunc = 0;
                    S.phase = PH_KICK_PICK;
                }
            }
            __syncwarp();
            cov_bar();
            return;
        }
        if (ph == PH_KICK_PICK) {
            if (tid == 0) {
                S.unc += (long long)S.acc.dunc;
                // the -1 ball appended newly uncovered words to the list
                const int cnt = cov_ldcg(&d.st->ul_n);
                if (S.ul_valid && cnt > d.ul_cap) S.ul_valid = 0;
                S.uln = min(cnt, d.ul_cap);
            }
            __syncwarp();
            cov_bar();
            long long w = leader_pick(d, S);
            if (tid == 0) {
                uint64_t pk;
                if (w >= 0) {
                    pk = pk_of_idx(d, (uint32_t)w);
                    for (int t2 = 0; t2 < d.R; t2++) {
                        // the value's draw precedes the position's draw, as
                        // the reference binary evaluates covsearch2e.c:1567
                        int val = (int)(rs_take(S) % (uint64_t)d.q);
                        int pos = (int)(rs_take(S) % (uint64_t)d.n);
                        pk = cov_setnib(pk, pos, val);
                    }
                } else {
                    pk = 0;
                    for (int j = 0; j < d.n; j++)
                        pk = cov_setnib(pk, j, (int)(rs_take(S) % (uint64_t)d.q));
                }
                OpParams &o = S.opp;
                leader_set_code(d, S, o.mi, pk);
                S.code_gen++;
                o.op = OP_BALL; o.sgn = +1; o.pc = pk; o.base = widx_pk(d, pk);
                o.ul_valid = S.ul_valid;
                S.acc.dunc = 0;
                S.phase = PH_KICK_RECOMP;
            }
            __syncwarp();
            cov_bar();
            return;
        }
        if (ph == PH_KICK_RECOMP) {
            if (tid == 0) {
                S.unc += (long long)S.acc.dunc;
                OpParams &o = S.opp;
                o.op = OP_RECOMPUTE;
                o.basen = o.base; o.pcn = o.pc;
                S.phase = PH_KICK_END;
            }
            __syncwarp();
            zero_acc(S);
            cov_bar();
            return;
        }
        if (ph == PH_KICK_END) {
            if (tid == 0) {
                const OpParams &o = S.opp;
                int32_t *Pk = d.P + (size_t)o.mi * (d.n + 1);
                cov_stcg(&Pk[0], S.acc.accT);
                for (int j = 0; j < d.n; j++) cov_stcg(&Pk[1 + j], S.acc.accH[j]);
                S.kick_t++;
                S.phase = PH_KICK_START;
            }
            __syncwarp();
            continue;
        }
        if (ph == PH_KICK_DONE) {
            if (tid == 0) {
                S.nkicks++;
                S.since_improve = 0;
                S.rec.kicked = 1;
                S.rec.unc_end = S.unc;
                S.rec.best = S.best_unc;
                write_trace(d, S);
                S.phase = PH_PLAN;
            }
            __syncwarp();
            continue;
        }
        if (ph == PH_GREEDY) {
            // greedy placement on uncovered words: covsearch2e.c:1210-1234
            if (S.greedy_i >= d.M) {
                if (tid == 0) { S.opp.op = OP_STOP; S.phase = PH_STOPPED; }
                __syncwarp();
                cov_bar();
                return;
            }
            long long w = leader_pick(d, S);
            if (tid == 0) {
                if (w < 0) w = (long long)(rs_take(S) % (uint64_t)d.N);
                uint64_t pk = pk_of_idx(d, (uint32_t)w);
                int i = S.greedy_i;
                leader_set_code(d, S, i, pk);
                S.code_gen++;
                OpParams &o = S.opp;
                o.op = OP_BALL; o.sgn = +1; o.mi = i; o.pc = pk; o.base = (uint32_t)w;
                o.ul_valid = 0;
                S.acc.dunc = 0;
                S.phase = PH_GREEDY_NEXT;
            }
            __syncwarp();
            cov_bar();
            return;
        }
        if (ph == PH_GREEDY_NEXT) {
            if (tid == 0) {
                S.unc += (long long)S.acc.dunc;
                S.greedy_i++;
                S.phase = PH_GREEDY;
            }
            __syncwarp();
            continue;
        }
        if (tid == 0) { S.status = COV_EDRIFT; S.opp.op = OP_STOP; S.phase = PH_STOPPED; }
        __syncwarp();
        cov_bar();
        return;
    }
    if (tid == 0) { S.status = COV_EDRIFT; S.opp.op = OP_STOP; S.phase = PH_STOPPED; }
    __syncwarp();
    cov_bar();
}

// ------------------------------------------------------------- kernel -----
// One instantiation per private-count upkeep form (per-lane or warp-
// aggregated commit), so that each is register-allocated on its own; a slot
// runs in the one its adjust mode names.
//
// help_ctas > 0 (one slot, gh set): the clusters after the first are helper
// CTAs of the first cluster's slot.  Each move's commit is then shared by
// every CTA of the grid: the search cluster publishes the move in gh, the
// helpers poll for it, take their share, add their sums to gh->acc and count
// themselves done; the leader waits for them (every wait is bounded by the
// launch deadline) before it reads the sums.
template <bool WARP>
__global__ void __launch_bounds__(NT, 1)
cov_run_kernel(const CovSlot *__restrict__ slots, const int *__restrict__ cluster_slot, int mode,
               unsigned long long budget_ns, long long op_guard, GridHelp *gh, int help_ctas)
{
    extern __shared__ __align__(16) unsigned char cov_smem[];
    Smem &S = *reinterpret_cast<Smem *>(cov_smem);
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int csize = (int)cl.num_blocks();
    const int cid = blockIdx.x / csize;
    const bool helper = help_ctas > 0 && cid > 0;
    if (threadIdx.x == 0) S.slot = slots[cluster_slot[helper ? 0 : cid]];
    __syncwarp();
    cov_bar();
    const CovSlot &d = S.slot;
    if (threadIdx.x == 0) { S.code_cached = d.M <= CODE_SM; S.code_gen = 0; }
    if (helper && __ldcg(&gh->absent)) return;
    if (helper) {
        // the code mirror: loaded here, then each shared move applied and
        // the whole code reloaded after other changes (kicks)
        if (d.M <= CODE_SM)
            for (int i = threadIdx.x; i < d.M; i += NT) S.code_sm[i] = cov_ldcg(&d.code[i]);
        cov_bar();
        const unsigned long long dl = (unsigned long long)cov_clock() +
                                      (budget_ns + 1000000000ull) * COV_CYCLES_PER_NS;
        unsigned seen = 0;
        for (;;) {
            if (threadIdx.x == 0) {
                int got = 0;
                // stop first: a helper that starts after the search cluster
                // has left must not replay the last move
                for (;;) {
                    if (ld_acquire_u32((const unsigned *)&gh->stop)) break;
                    const unsigned sq = ld_acquire_u32(&gh->seq);
                    if (sq != seen) { seen = sq; got = 1; break; }
                    if ((unsigned long long)cov_clock() > dl) { set_error(d, COV_ETIMEOUT); break; }
                    __nanosleep(64);
                }
                if (got) {
                    const unsigned *src = reinterpret_cast<const unsigned *>(&gh->op);
                    unsigned *dst = reinterpret_cast<unsigned *>(&S.opl);
                    for (int k = 0; k < (int)(sizeof(OpParams) / 4); k++) dst[k] = __ldcg(src + k);
                    const int cg = __ldcg(&gh->code_gen);
                    S.gh_reload = cg != S.code_gen;
                    S.code_gen = cg;
                }
                S.gh_got = got;
            }
            cov_bar();
            if (!S.gh_got) break;
            if (S.gh_reload && d.M <= CODE_SM) {
                for (int i = threadIdx.x; i < d.M; i += NT) S.code_sm[i] = cov_ldcg(&d.code[i]);
                cov_bar();
            }
            op_move_t<WARP>(d, S.opl, S, &gh->acc, (int)blockIdx.x, (int)gridDim.x, true);
            __threadfence();
            cov_bar();
            if (threadIdx.x == 0 && d.M <= CODE_SM) S.code_sm[S.opl.mi] = S.opl.pcn;
            if (threadIdx.x == 0) atomicAdd(&gh->done, 1u);
        }
        return;
    }
    const bool leader = rank == 0;
    Smem *LS = cl.map_shared_rank(&S, 0);

    if (leader)
        for (int m = threadIdx.x; m <= INV_N; m += NT)
            S.inv[m] = m ? 0xffffffffffffffffull / (uint64_t)m : 0;
    if (d.M <= CODE_SM)
        for (int i = threadIdx.x; i < d.M; i += NT) S.code_sm[i] = cov_ldcg(&d.code[i]);
    if (leader && threadIdx.x == 0) {
        CovSlotState *st = d.st;
        rs_init(S, st->rng);
        S.it = st->it; S.unc = st->unc; S.best_unc = st->best_unc;
        S.since_improve = st->since_improve; S.nkicks = st->nkicks;
        S.moves_left = st->moves_left; S.target = st->target; S.trace_n = st->trace_n;
        S.ul_valid = st->ul_valid; S.status = st->status; S.finished = st->finished;
        S.mode = mode;
        S.greedy_i = (int)st->moves_left;   // greedy: first codeword to place
        S.phase = PH_PLAN;
        S.t_deadline = (unsigned long long)cov_clock() + budget_ns * COV_CYCLES_PER_NS;
        S.guard = 0;
        S.opp.op = -1;
        S.gh_seq = 0;
        S.code_gen = 0;
        S.noisy = 0;
        S.sa_accept = 0;
        S.sa_T = st->sa_T;
        for (int k = 0; k < 24; k++) S.prof[k] = st->prof[k];
        S.ul_pairs = st->stat_ul_pairs;
    }
    cov_cbar(cl);
    for (;;) {
        if (leader) {
            leader_step(d, S, csize);
            // safety net: an op budget and the launch deadline bound every
            // launch even if the phase machine never reaches a move boundary
            if (threadIdx.x == 0 && S.opp.op != OP_STOP &&
                (++S.guard > op_guard ||
                 (unsigned long long)cov_clock() > S.t_deadline + 1000000000ull * COV_CYCLES_PER_NS)) {
                S.status = COV_ETIMEOUT;
                S.opp.op = OP_STOP;
                S.phase = PH_STOPPED;
            }
        }
        cov_cbar(cl);
        if (threadIdx.x == 0) S.opl = LS->opp;
        __syncwarp();
        cov_bar();
        const OpParams &P = S.opl;
        const int op = P.op;
        if (op == OP_STOP) break;
        const long long top = cov_clock();
        const bool shared_move = op == OP_MOVE && help_ctas > 0;
        if (shared_move && leader && threadIdx.x == 0) {
            // publish the move to the helpers (they are all done with the last one)
            gh->done = 0;
            gh->code_gen = S.code_gen;
            const unsigned *src = reinterpret_cast<const unsigned *>(&P);
            unsigned *dst = reinterpret_cast<unsigned *>(&gh->op);
            for (int k = 0; k < (int)(sizeof(OpParams) / 4); k++) dst[k] = src[k];
            st_release_u32(&gh->seq, ++S.gh_seq);
        }
        if (op == OP_MOVE) {
            op_move_t<WARP>(d, P, S, &LS->acc, rank, csize + help_ctas, help_ctas > 0);
            if (d.M <= CODE_SM && threadIdx.x == 0) S.code_sm[P.mi] = P.pcn;
        } else if (op == OP_NEGWALK) {
            op_negwalk<WARP>(d, P, S, LS, rank, csize, cl);
        } else if (op == OP_NEG) {
            op_neg(d, P, S, LS, rank, csize);
        } else if (op == OP_BALL) {
            // a +1 ball places the slot's new codeword: mirror it first
            if (P.sgn > 0 && d.M <= CODE_SM && threadIdx.x == 0) S.code_sm[P.mi] = P.pc;
            cov_bar();
            op_ball(d, P, LS, rank, csize);
        } else if (op == OP_RECOMPUTE) {
            op_recompute(d, P.basen, P.pcn, S, LS, rank, csize);
        } else if (op == OP_ZERO_TABU) {
            op_zero_tabu(d, rank, csize);
        } else if (op == OP_REBUILD_UL) {
            op_rebuild_ul(d, rank, csize, cl);
        }
        cov_cbar(cl);
        if (shared_move && leader) {
            // the helpers' share: wait for all of them, then add their sums
            if (threadIdx.x == 0) {
                bool ok = true;
                const long long tw = cov_clock();
                S.prof[15] += tw - top;
                while (ld_acquire_u32(&gh->done) < (unsigned)help_ctas) {
                    if ((unsigned long long)cov_clock() > S.t_deadline + 1000000000ull * COV_CYCLES_PER_NS) {
                        ok = false;
                        break;
                    }
                }
                S.prof[12] += cov_clock() - tw;
                if (ok) {
                    S.acc.dunc += __ldcg(&gh->acc.dunc);
                    S.acc.accT += __ldcg(&gh->acc.accT);
                    for (int j = 0; j < d.n; j++) S.acc.accH[j] += __ldcg(&gh->acc.accH[j]);
                    gh->acc.dunc = 0;
                    gh->acc.accT = 0;
                    for (int j = 0; j < d.n; j++) gh->acc.accH[j] = 0;
                } else {
                    // a helper never answered: its share of the move may be
                    // missing, so the state is no longer consistent
                    S.status = COV_EDRIFT;
                    S.phase = PH_STOPPED;
                }
            }
            cov_bar();
        }
        if (leader && threadIdx.x == 0) {
            const long long dt = cov_clock() - top;
            if (op == OP_MOVE) S.prof[4] += dt;
            else if (op == OP_NEGWALK || op == OP_NEG) { S.prof[2] += dt; S.prof[14] += dt; }
            else S.prof[7] += dt;
        }
    }
    // no CTA may leave while another can still read the leader's shared memory
    cov_cbar(cl);
    if (help_ctas > 0 && leader && threadIdx.x == 0) st_release_u32((unsigned *)&gh->stop, 1u);
    if (leader && threadIdx.x == 0) {
        CovSlotState *st = d.st;
        rs_final(S, st->rng);
        st->it = S.it; st->unc = S.unc; st->best_unc = S.best_unc;
        st->since_improve = S.since_improve; st->nkicks = S.nkicks;
        st->moves_left = S.moves_left; st->trace_n = S.trace_n;
        st->ul_valid = S.ul_valid;
        st->sa_T = S.sa_T;
        for (int k = 0; k < 24; k++) st->prof[k] = S.prof[k];
        st->stat_ul_pairs = S.ul_pairs;
        int s0 = atomicAdd(&st->status, 0);
        st->status = S.status ? S.status : s0;
        st->finished = S.unc <= 0;
    }
}

// ------------------------------------------------------ init kernels -------
// cnt|id-sum marking of the balls of codewords first..first+count-1 (the
// incremental form, used by greedy placement and remove-and-repair)
__global__ void k_mark_balls(CovSlot d, int first, int count, int sgn)
{
    const int R = d.R;
    uint32_t cum[COV_MAXN + 2];
    cum[0] = 1;
    for (int r = 1; r <= R; r++)
        cum[r] = cum[r - 1] + sphere_items(d, r, d.ball_off[r + 1] - d.ball_off[r]);
    const unsigned long long per = cum[R];
    const unsigned long long total = per * (unsigned long long)count;
    for (unsigned long long g = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; g < total;
         g += (unsigned long long)gridDim.x * blockDim.x) {
        const int i = first + (int)(g / per);
        const uint32_t t = (uint32_t)(g - (unsigned long long)(i - first) * per);
        const uint64_t pc = d.code[i];
        const uint32_t base = widx_pk(d, pc);
        const uint32_t add = sgn > 0 ? cov_cw_unit(i) : 0u - cov_cw_unit(i);
        if (t == 0) { atomicAdd(&d.cw[base], add); continue; }
        int r = 1;
        while (t >= cum[r]) r++;
        const uint8_t *subs = d.ball_sub + (size_t)d.ball_off[r] * d.rs;
        CovItem it = cov_item(d, subs, r, t - cum[r - 1], base, pc);
        for (int kk = 0; kk < d.q - 1; kk++) {
            uint32_t w; uint64_t pk;
            cov_item_word(d, it, kk, w, pk);
            atomicAdd(&d.cw[w], add);
        }
    }
}

// Whole-state build, one CTA per tile of q^bt_nl consecutive words (the
// words sharing their first bt_nh digits; cov_tiles.cuh marks the balls):
// each covered word gets 1 + (id << 16) per coverer, and the tile's
// counters are written to HBM once.
// Before leaving, the CTA counts the tile's uncovered words (zeros[0]),
// appends them to the uncovered-word list (zeros[1] counts the appends; the
// list is complete if that stays within its capacity -- the rebuild of
// covsearch2e.c:323-338 done in the same pass), and adds each singly covered
// word at distance exactly R from its coverer k to P[k] = (T_k, H_k) -- the
// counts the reference's shared-sphere walk (covsearch2e.c:592-654)
// produces for k.  ul_bit must be clear beforehand.

template <int Q>
__global__ void __launch_bounds__(BT_NT) k_build_state(CovSlot d, unsigned long long *zeros)
{
    extern __shared__ __align__(16) unsigned char bt_raw[];
    uint64_t *lpc = (uint64_t *)bt_raw;            // [BT_LCH] packed codewords of this chunk
    uint32_t *lid = (uint32_t *)(lpc + BT_LCH);    // [BT_LCH] their ids
    uint32_t *lbase = lid + BT_LCH;                // [BT_LCH] their low-digit index
    uint32_t *tile = lbase + BT_LCH;               // [bt_tw]
    __shared__ int gcnt[COV_MAXN + 2], gpos[COV_MAXN + 2], gfill[COV_MAXN + 2];

    const int q = d.q, n = d.n, R = d.R, nh = d.bt_nh, nl = d.bt_nl;
    const uint32_t T = d.bt_tw;
    uint64_t hp = 0;
    {
        uint32_t t = blockIdx.x;
        for (int j = nh - 1; j >= 0; --j) { hp |= (uint64_t)(t % (uint32_t)q) << (4 * j); t /= (uint32_t)q; }
    }
    for (uint32_t x = threadIdx.x; x < T; x += BT_NT) tile[x] = 0;
    BtScratch sc{lpc, lid, lbase, gcnt, gpos, gfill};
    bt_mark_tile<Q>(tile, d.q, d.n, R, d.M, d.code, d.pw, nh, nl, d.bt_items, d.bt_last, d.bt_v, hp, sc,
                    [](uint32_t id) { return cov_cw_unit((int)id); });

    uint32_t *gout = d.cw + (size_t)blockIdx.x * T;
    unsigned long long z = 0;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (uint32_t x0 = 0; x0 < T; x0 += BT_NT) {
        const uint32_t x = x0 + threadIdx.x;
        const bool in = x < T;
        const uint32_t v = in ? tile[x] : 1u;
        const uint32_t c = v & 0xffffu;
        uint64_t pk = hp;
        if (in) {
            gout[x] = v;
            uint32_t y = x;
            if (c <= 1)
                for (int j = n - 1; j >= nh; --j) { pk |= (uint64_t)(y % (uint32_t)q) << (4 * j); y /= (uint32_t)q; }
        }
        // uncovered words go on the uncovered-word list (order is free: the
        // list only feeds sums and the first-after-start search)
        const bool zero = in && c == 0;
        const unsigned zm = __ballot_sync(FULL, zero);
        if (zm) {
            unsigned long long base = 0;
            if (lane == __ffs(zm) - 1) base = atomicAdd(&zeros[1], (unsigned long long)__popc(zm));
            base = __shfl_sync(FULL, base, __ffs(zm) - 1);
            if (zero) {
                const unsigned long long at = base + __popc(zm & ((1u << lane) - 1));
                const uint32_t gx = blockIdx.x * T + x;
                if (at < (unsigned long long)d.ul_cap) {
                    d.ul_idx[at] = gx;
                    d.ul_pk[at] = pk;
                    atomicOr(&d.ul_bit[gx >> 5], 1u << (gx & 31));
                }
                if (d.zbits) atomicOr(&d.zb[gx >> 5], 1u << (gx & 31));
            }
        }
        z += zero;
        if (in && c == 1) {
            const int k = (int)(v >> 16);
            uint64_t D = cov_spread(pk ^ d.code[k]);
            if (__popcll(D) == R) {
                int32_t *Pk = d.P + (size_t)k * (n + 1);
                atomicAdd(&Pk[0], 1);
                while (D) {
                    const int j = (__ffsll((long long)D) - 1) >> 2;
                    D &= D - 1;
                    atomicAdd(&Pk[1 + j], 1);
                }
            }
        }
    }
    z = warp_sum(z);
    if ((threadIdx.x & 31) == 0 && z) atomicAdd(zeros, z);
}

__global__ void k_count_zero(const uint32_t *cw, uint32_t N, unsigned long long *out)
{
    unsigned long long c = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        c += (cw[x] & 0xffffu) == 0;
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// words of codeword i's ball that nothing else covers (covsearch2e.c:927-946)
__global__ void k_unique_cover(CovSlot d, int count, int *out)
{
    const int R = d.R;
    const int i = blockIdx.x;
    if (i >= count) return;
    uint32_t cum[COV_MAXN + 2];
    cum[0] = 1;
    for (int r = 1; r <= R; r++)
        cum[r] = cum[r - 1] + sphere_items(d, r, d.ball_off[r + 1] - d.ball_off[r]);
    const uint64_t pc = d.code[i];
    const uint32_t base = widx_pk(d, pc);
    int u = 0;
    for (uint32_t t = threadIdx.x; t < cum[R]; t += blockDim.x) {
        if (t == 0) { u += (d.cw[base] & 0xffffu) == 1; continue; }
        int r = 1;
        while (t >= cum[r]) r++;
        const uint8_t *subs = d.ball_sub + (size_t)d.ball_off[r] * d.rs;
        CovItem it = cov_item(d, subs, r, t - cum[r - 1], base, pc);
        for (int kk = 0; kk < d.q - 1; kk++) {
            uint32_t w; uint64_t pk;
            cov_item_word(d, it, kk, w, pk);
            u += (d.cw[w] & 0xffffu) == 1;
        }
    }
    __shared__ int red[32];
    u = warp_sum(u);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = u;
    cov_bar();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) s += red[w];
        out[i] = s;
    }
    __syncwarp();
}

// per-launch budget of every listed slot, set on the device so that a run
// needs no host round trip (and can be captured in a graph)
__global__ void k_set_budget(CovSlotState *states, const int *map, int nslots, long long moves,
                             long long target)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nslots) {
        CovSlotState &s = states[map[k]];
        long long m = moves;
        if (s.it_limit >= 0) m = min(m, max(0ll, s.it_limit - s.it));
        s.moves_left = m;
        s.target = target;
    }
}

__global__ void k_unpack_cnt(const uint32_t *cw, uint32_t N, uint16_t *out)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        out[x] = (uint16_t)(cw[x] & 0xffffu);
}

// =========================================================== host side =====
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "covgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    return -(100 + (int)e_); } } while (0)

namespace {

long long ipow_h(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }
long long binom_h(int a, int b)
{
    if (b < 0 || b > a) return 0;
    if (b > a - b) b = a - b;
    long long r = 1;
    for (int i = 0; i < b; i++) r = r * (a - i) / (i + 1);
    return r;
}

// Private-count events of a commit (words crossing multiplicity 1 <-> 2):
// with mean coverage lambda = M |B| / q^n -- fixed for an instance, the sum
// of all counts being M |B| -- about 2 S' lambda e^-lambda (1 + lambda/2)
// per move.  From ~8k per move the warp-aggregated form is the faster one.
static int padj_auto(int q, int n, int R, int M)
{
    if (R < 1 || R >= n) return 0;
    double V = 0;
    for (int r = 0; r <= R; r++) V += (double)binom_h(n, r) * (double)ipow_h(q - 1, r);
    const double lam = (double)M * V / (double)ipow_h(q, n);
    const double Sp = (double)binom_h(n - 1, R) * (double)ipow_h(q - 1, R);
    return 2.0 * Sp * lam * std::exp(-lam) * (1.0 + lam / 2.0) >= 8192.0;
}

int fill_subsets_h(const int *pool, int np, int R, int rs, uint8_t *out)
{
    if (binom_h(np, R) <= 0) return 0;
    int c[32], k = 0;
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

struct HostSlot {
    bool used = false;
    CovSlot d{};
    CovSlotState *st = nullptr;
    void *arena = nullptr;       // one device allocation for all arrays
    size_t arena_bytes = 0;
    int cluster = 1;
    int cap = 0;                 // codewords the storage holds
    cov_params prm{};
};

}  // namespace

struct cov_pool {
    int max_slots = 0;
    int cluster = 8;
    std::vector<HostSlot> slots;
    CovSlot *d_slots = nullptr;
    int *d_map = nullptr;            // scratch list for single-slot launches
    int *d_all = nullptr;            // every used slot
    int n_all = 0;
    bool all_dirty = true;
    CovSlotState *d_states = nullptr;
    cudaStream_t stream = nullptr;   // the pool's own stream
    cudaStream_t ext = nullptr;      // caller's stream, when set
    bool use_ext = false;
    double budget_s = 30.0;
    long long launch_moves = 0;      // move budget of the current launch
    long long neg_cluster_pairs = NEG_CLUSTER_PAIRS;
    int list_cost = LIST_COST;
    cudaGraphExec_t gexec = nullptr; // captured multi-step run
    long long g_moves = -1, g_target = -2;
    int g_steps = 0;
    // slots grouped by cluster size: d_all holds the groups one after the
    // other; every group after the first runs on its own stream, forked from
    // and joined back to the current stream
    struct Group { int csize, warp, off, count; };
    std::vector<Group> groups;
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> ev;      // ev[0] fork, ev[1 + g] join of group g
    // a pool with one slot: its moves' commits shared with helper CTAs on
    // the SMs its cluster leaves free (0 off, else the most helper clusters)
    int grid_help = 0;
    int grid_help_absent = 0;        // test setting (GridHelp::absent)
    GridHelp *d_gh = nullptr;
    int help_clusters[17][2] = {};    // co-resident clusters - 1, per cluster size and form (+1: known)
    cudaStream_t cur_stream() const { return use_ext ? ext : stream; }
};

static CovDeviceFlags g_attr_done;   // kernel attributes set, per device

static int ensure_attrs()
{
    int dev = 0;
    if (g_attr_done.done(dev)) return 0;
    CK(cudaFuncSetAttribute(cov_run_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem)));
    CK(cudaFuncSetAttribute(cov_run_kernel<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    CK(cudaFuncSetAttribute(cov_run_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem)));
    CK(cudaFuncSetAttribute(cov_run_kernel<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    CK(cudaFuncSetAttribute(k_build_state<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt_smem_bytes(BT_MAX)));
#define BS_ATTR_Q(QQ) \
    CK(cudaFuncSetAttribute(k_build_state<QQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt_smem_bytes(BT_MAX)));
    BT_Q_LIST(BS_ATTR_Q)
#undef BS_ATTR_Q
    g_attr_done.set(dev);
    return 0;
}

// helper clusters for a one-slot search at cluster size csize: as many as
// can be resident beside the search cluster, at most pool->grid_help
static int help_clusters(cov_pool *pool, int csize, int warp, int *out)
{
    *out = 0;
    int &c = pool->help_clusters[csize][warp];
    if (!c) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)csize);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = sizeof(Smem);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)csize;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nc = 0;
        CK(cudaOccupancyMaxActiveClusters(&nc, warp ? cov_run_kernel<true> : cov_run_kernel<false>, &cfg));
        c = 1 + std::max(0, nc - 1);
    }
    *out = std::min(c - 1, pool->grid_help);
    return 0;
}

// one cluster per listed slot; d_list holds `count` slot indices on the device
static int launch_kernel(cov_pool *pool, const int *d_list, int count, int csize, int warp, int mode,
                         long long moves, cudaStream_t stream)
{
    if (count <= 0) return 0;
    int help = 0;
    if (pool->grid_help > 0 && count == 1 && pool->n_all == 1 && mode == MODE_SEARCH) {
        int rc = help_clusters(pool, csize, warp, &help);
        if (rc) return rc;
    }
    const int help_ctas = help * csize;
    if (help_ctas) {
        CK(cudaMemsetAsync(pool->d_gh, 0, sizeof(GridHelp), stream));
        if (pool->grid_help_absent)
            CK(cudaMemcpyAsync(&pool->d_gh->absent, &pool->grid_help_absent, sizeof(int), cudaMemcpyHostToDevice,
                               stream));
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(count * csize + help_ctas));
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = sizeof(Smem);
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    unsigned long long budget_ns = (unsigned long long)(pool->budget_s * 1e9);
    // ops per move <= 2 (walk + move) + a kick's 3 per codeword + 2
    int kmax = 0;
    long long mmax = 0;
    for (int s = 0; s < pool->max_slots; s++) {
        if (!pool->slots[s].used) continue;
        kmax = std::max(kmax, pool->slots[s].d.kick);
        mmax = std::max<long long>(mmax, pool->slots[s].d.M);
    }
    long long guard = mode == MODE_GREEDY ? 4 * mmax + 4096 : moves * (6 + 3LL * kmax) + 4096;
    CK(cudaLaunchKernelEx(&cfg, warp ? cov_run_kernel<true> : cov_run_kernel<false>,
                          (const CovSlot *)pool->d_slots, d_list, mode, budget_ns,
                          guard, pool->d_gh, help_ctas));
    CK(cudaGetLastError());
    return 0;
}

// launch for an explicit host list of slots (initialisation paths)
static int launch_run(cov_pool *pool, const std::vector<int> &active, int csize, int mode)
{
    if (active.empty()) return 0;
    CK(cudaMemcpyAsync(pool->d_map, active.data(), sizeof(int) * active.size(), cudaMemcpyHostToDevice,
                       pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    int warp = 0;
    for (int s : active) warp |= pool->slots[s].d.padj_warp;
    return launch_kernel(pool, pool->d_map, (int)active.size(), csize, warp, mode, pool->launch_moves,
                         pool->cur_stream());
}

// device list of every used slot, refreshed after add/remove
static int refresh_all(cov_pool *pool)
{
    if (!pool->all_dirty) return 0;
    std::vector<int> all;
    pool->groups.clear();
    for (int c = 1; c <= 16; c++) {
        for (int w = 0; w < 2; w++) {
            const int off = (int)all.size();
            for (int s = 0; s < pool->max_slots; s++)
                if (pool->slots[s].used && pool->slots[s].cluster == c && pool->slots[s].d.padj_warp == w)
                    all.push_back(s);
            if ((int)all.size() > off) pool->groups.push_back({c, w, off, (int)all.size() - off});
        }
    }
    if (!all.empty())
        CK(cudaMemcpy(pool->d_all, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice));
    while (pool->aux.size() + 1 < pool->groups.size()) {
        cudaStream_t a;
        CK(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
        pool->aux.push_back(a);
    }
    while (pool->ev.size() < pool->groups.size() + 1) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        pool->ev.push_back(e);
    }
    pool->n_all = (int)all.size();
    pool->all_dirty = false;
    if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
    return 0;
}

// budget + run for every used slot, enqueued on the current stream (groups
// of other cluster sizes on forked streams that join back into it)
static int enqueue_step(cov_pool *pool, long long moves, long long target)
{
    if (pool->n_all == 0) return 0;
    cudaStream_t st = pool->cur_stream();
    k_set_budget<<<(pool->n_all + 127) / 128, 128, 0, st>>>(pool->d_states, pool->d_all, pool->n_all, moves,
                                                            target);
    CK(cudaGetLastError());
    const int ng = (int)pool->groups.size();
    if (ng > 1) CK(cudaEventRecord(pool->ev[0], st));
    for (int g = 1; g < ng; g++) {
        const cov_pool::Group &G = pool->groups[g];
        cudaStream_t a = pool->aux[g - 1];
        CK(cudaStreamWaitEvent(a, pool->ev[0], 0));
        int rc = launch_kernel(pool, pool->d_all + G.off, G.count, G.csize, G.warp, MODE_SEARCH, moves, a);
        if (rc) return rc;
        CK(cudaEventRecord(pool->ev[1 + g], a));
    }
    const cov_pool::Group &G0 = pool->groups[0];
    int rc = launch_kernel(pool, pool->d_all + G0.off, G0.count, G0.csize, G0.warp, MODE_SEARCH, moves, st);
    if (rc) return rc;
    for (int g = 1; g < ng; g++) CK(cudaStreamWaitEvent(st, pool->ev[1 + g], 0));
    return 0;
}

static int push_slot(cov_pool *pool, int s)
{
    CK(cudaMemcpyAsync(pool->d_slots + s, &pool->slots[s].d, sizeof(CovSlot), cudaMemcpyHostToDevice,
                       pool->cur_stream()));
    return 0;
}

static int read_state(cov_pool *pool, int s, CovSlotState *out)
{
    CK(cudaMemcpyAsync(out, pool->slots[s].st, sizeof(CovSlotState), cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return 0;
}


extern "C" {

int cov_pool_create(int32_t max_slots, int32_t cluster, cov_pool **out)
{
    if (!out || max_slots < 1 || cluster < 1 || cluster > 16) return COV_EINVAL;
    *out = nullptr;
    int dev = 0, major = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major < 10) return COV_ENODEV;
    int rc = ensure_attrs();
    if (rc) return rc;
    cov_pool *p = new cov_pool();
    p->max_slots = max_slots;
    p->cluster = cluster;
    p->slots.resize(max_slots);
    if (cudaMalloc(&p->d_slots, sizeof(CovSlot) * max_slots) != cudaSuccess ||
        cudaMalloc(&p->d_map, sizeof(int) * max_slots) != cudaSuccess ||
        cudaMalloc(&p->d_all, sizeof(int) * max_slots) != cudaSuccess ||
        cudaMalloc(&p->d_states, sizeof(CovSlotState) * max_slots) != cudaSuccess) {
        cudaFree(p->d_slots); cudaFree(p->d_map); cudaFree(p->d_all); cudaFree(p->d_states);
        delete p;
        return COV_ENOMEM;
    }
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaFree(p->d_slots); cudaFree(p->d_map); cudaFree(p->d_states);
        delete p;
        return COV_ENOMEM;
    }
    *out = p;
    return COV_OK;
}

int cov_pool_set_budget(cov_pool *pool, double seconds)
{
    if (!pool || !(seconds > 0)) return COV_EINVAL;
    pool->budget_s = seconds;
    return COV_OK;
}

// A slot stopped by its launch deadline (COV_ETIMEOUT) stopped between two
// moves with its state whole: clear the status so that the next run goes on
// from there, on exactly the trajectory an uninterrupted run follows.  Any
// other error stays.
int cov_pool_resume(cov_pool *pool, int32_t slot)
{
    if (!pool || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    CovSlotState hs;
    int rc = read_state(pool, slot, &hs);
    if (rc) return rc;
    if (hs.status == COV_OK) return COV_OK;
    if (hs.status != COV_ETIMEOUT) return hs.status;
    int zero = 0;
    CK(cudaMemcpyAsync(&pool->slots[slot].st->status, &zero, sizeof zero, cudaMemcpyHostToDevice,
                       pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return COV_OK;
}

int cov_pool_remove(cov_pool *pool, int32_t slot)
{
    if (!pool || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    HostSlot &h = pool->slots[slot];
    cudaStreamSynchronize(pool->cur_stream());
    cudaFree(h.arena);
    h = HostSlot();
    pool->all_dirty = true;
    return COV_OK;
}

int cov_pool_destroy(cov_pool *pool)
{
    if (!pool) return COV_OK;
    cudaStreamSynchronize(pool->cur_stream());
    for (int s = 0; s < pool->max_slots; s++)
        if (pool->slots[s].used) cudaFree(pool->slots[s].arena);
    if (pool->gexec) cudaGraphExecDestroy(pool->gexec);
    cudaFree(pool->d_slots); cudaFree(pool->d_map); cudaFree(pool->d_all); cudaFree(pool->d_states);
    cudaFree(pool->d_gh);
    for (cudaStream_t a : pool->aux) cudaStreamDestroy(a);
    for (cudaEvent_t e : pool->ev) cudaEventDestroy(e);
    cudaStreamDestroy(pool->stream);
    delete pool;
    return COV_OK;
}

size_t cov_slot_bytes(const cov_params *prm)
{
    if (!prm) return 0;
    const int q = prm->q, n = prm->n, R = prm->R, M = prm->M;
    if (q < 2 || q > 16 || n < 1 || n > 16 || R < 0 || M < 1 || M > 65535) return 0;
    long long N = ipow_h(q, n);
    size_t b = 0;
    auto add = [&](size_t x) { b += (x + 255) / 256 * 256; };
    add((size_t)N * 4);                              // cw
    add((size_t)M * 8 * 2);                          // code, best
    add((size_t)M * n * q * 4);                      // tabu
    add((size_t)M * (n + 1) * 4);                    // P
    add((size_t)UL_CAP_DEFAULT * 4);                 // ul_idx
    add((size_t)UL_CAP_DEFAULT * 8);                 // ul_pk
    add((size_t)((N + 31) / 32) * 4);                // ul_bit
    add((size_t)((N + 31) / 32) * 4);                // zb
    const size_t ce = (size_t)M * n * (prm->wide ? (size_t)(q - 1) : 1u);
    add(ce * 4 * 2 + (size_t)M * n * 4 + (size_t)M * 4);   // g_perm, g_dval, g_neg, g_list
    if (prm->wide) add((size_t)M * n * q * 4);      // g_negw
    add(65536);                                      // subset tables
    {
        int nh, nl;
        bt_geom(q, n, &nh, &nl);
        uint32_t vc[COV_MAXN + 2];
        std::vector<uint8_t> lst;
        const size_t ni = bt_items_h(q, n, std::min(R, n), nh, vc, lst).size();
        add(ni * 8);                                 // state-build ball groups
        add(ni);
    }
    add(sizeof(CovSlotState));
    if (prm->trace) add((size_t)prm->trace_cap * sizeof(cov_move_rec));
    return b;
}

// Allocate slot storage for up to `cap` codewords (cap >= M; remove-and-
// repair needs the whole oversized seed) and fill the descriptor.
static int slot_alloc(cov_pool *pool, const cov_params *prm, int cap, int *s_out)
{
    const int q = prm->q, n = prm->n, M = prm->M;
    int R = prm->R;
    if (q < 2 || q > 16 || n < 1 || n > 16 || R < 0 || M < 1 || M > 65535) return COV_EINVAL;
    if (prm->cand < 1 || prm->kick < 0 || prm->stall < 0 || prm->trace_cap < 0) return COV_EINVAL;
    if (cap > 65535) return COV_ERANGE;
    long long N = ipow_h(q, n);
    if (N >= (1LL << 32) - 1) return COV_EINVAL;
    if (prm->wide < 0 || prm->wide > 1) return COV_EINVAL;
    if (prm->fix0 < 0 || prm->fix0 > 1 || (prm->fix0 && prm->M < 2)) return COV_EINVAL;
    if (prm->sa < 0 || prm->sa > 1) return COV_EINVAL;
    if (R > n) R = n;
    int s = -1;
    for (int k = 0; k < pool->max_slots; k++) if (!pool->slots[k].used) { s = k; break; }
    if (s < 0) return COV_ERANGE;
    const int Mw = std::max(M, cap);

    HostSlot h;
    h.prm = *prm;
    h.cluster = pool->cluster;
    h.cap = Mw;
    CovSlot &d = h.d;
    d.q = q; d.n = n; d.R = R; d.M = M;
    d.N = (uint32_t)N;
    for (int j = 0; j < n; j++) d.pw[j] = (uint32_t)ipow_h(q, n - 1 - j);
    d.rs = R ? R : 1;
    d.nsub = (int)binom_h(n - 1, R);
    d.nfsub = (int)binom_h(n, R);
    for (int k = 0; k <= COV_MAXN; k++) d.ppow[k] = (uint32_t)std::min<long long>(ipow_h(q - 1, k), 0xffffffffLL);
    d.tenure = prm->tabu; d.kick = prm->kick; d.cand = prm->cand; d.stall = prm->stall;
    d.ul_cap = UL_CAP_DEFAULT;
    d.neg_cluster_pairs = pool->neg_cluster_pairs;
    d.list_cost = pool->list_cost;
    d.wide = prm->wide ? 1 : 0;
    d.fix0 = prm->fix0 ? 1 : 0;
    d.sa = prm->sa ? 1 : 0;
    d.noise = prm->noise;
    d.sa_t0 = prm->t0;
    d.sa_cool = prm->cool;
    d.sa_tmin = prm->tmin;
    d.wide_sliced = 1;
    d.padj_warp = padj_auto(q, n, R, M);
    d.zbits = d.padj_warp;
    std::vector<uint8_t> subs((size_t)n * std::max(d.nsub, 1) * d.rs, 0);
    for (int p = 0; p < n; p++) {
        int pool_[32], np = 0;
        for (int j = 0; j < n; j++) if (j != p) pool_[np++] = j;
        fill_subsets_h(pool_, np, R, d.rs, subs.data() + (size_t)p * d.nsub * d.rs);
    }
    d.nsub1 = R >= 1 ? (int)binom_h(n - 1, R - 1) : 0;
    std::vector<uint8_t> subs1((size_t)n * std::max(d.nsub1, 1) * d.rs, 0);
    if (R >= 2) {
        for (int p = 0; p < n; p++) {
            int pool_[32], np = 0;
            for (int j = 0; j < n; j++) if (j != p) pool_[np++] = j;
            fill_subsets_h(pool_, np, R - 1, d.rs, subs1.data() + (size_t)p * d.nsub1 * d.rs);
        }
    }
    std::vector<uint8_t> balls;
    {
        int pool_[32];
        for (int j = 0; j < n; j++) pool_[j] = j;
        int off = 0;
        for (int r = 0; r <= R; r++) {
            d.ball_off[r] = off;
            int cnt = (int)binom_h(n, r);
            balls.resize((size_t)(off + cnt) * d.rs, 0);
            if (r > 0) fill_subsets_h(pool_, n, r, d.rs, balls.data() + (size_t)off * d.rs);
            off += cnt;
        }
        d.ball_off[R + 1] = off;
    }
    cov_params p2 = *prm;
    p2.M = Mw;
    size_t need = cov_slot_bytes(&p2) + subs.size() + subs1.size() + balls.size() + 2048;
    void *arena = nullptr;
    if (cudaMalloc(&arena, need) != cudaSuccess) { cudaGetLastError(); return COV_ENOMEM; }
    size_t off = 0;
    auto take_ = [&](size_t x) { void *p = (char *)arena + off; off += (x + 255) / 256 * 256; return p; };
    d.cw = (uint32_t *)take_((size_t)N * 4);
    d.code = (uint64_t *)take_((size_t)Mw * 8);
    d.best = (uint64_t *)take_((size_t)Mw * 8);
    d.tabu = (int32_t *)take_((size_t)Mw * n * q * 4);
    d.P = (int32_t *)take_((size_t)Mw * (n + 1) * 4);
    d.ul_idx = (uint32_t *)take_((size_t)d.ul_cap * 4);
    d.ul_pk = (uint64_t *)take_((size_t)d.ul_cap * 8);
    d.ul_bit = (uint32_t *)take_((size_t)((N + 31) / 32) * 4);
    d.zb = (uint32_t *)take_((size_t)((N + 31) / 32) * 4);
    const size_t ce = (size_t)Mw * n * (prm->wide ? (size_t)(q - 1) : 1u);
    d.g_perm = (uint32_t *)take_(ce * 4);
    d.g_dval = (int32_t *)take_(ce * 4);
    d.g_neg = (int32_t *)take_((size_t)Mw * n * 4);
    d.g_list = (uint32_t *)take_((size_t)Mw * 4);
    d.g_negw = prm->wide ? (int32_t *)take_((size_t)Mw * n * q * 4) : nullptr;
    uint8_t *dsub = (uint8_t *)take_(subs.size());
    uint8_t *dball = (uint8_t *)take_(balls.size());
    uint8_t *dsub1 = (uint8_t *)take_(subs1.size());
    d.sub = dsub; d.ball_sub = dball; d.sub1 = dsub1;
    bt_geom(q, n, &d.bt_nh, &d.bt_nl);
    d.bt_tw = (uint32_t)ipow_h(q, d.bt_nl);
    std::vector<uint8_t> btl;
    std::vector<uint64_t> bti = bt_items_h(q, n, R, d.bt_nh, d.bt_v, btl);
    uint64_t *dbt = (uint64_t *)take_(bti.size() * 8);
    uint8_t *dbl = (uint8_t *)take_(btl.size());
    d.bt_items = dbt;
    d.bt_last = dbl;
    d.st = pool->d_states + s;
    d.trace = prm->trace ? take_((size_t)prm->trace_cap * sizeof(cov_move_rec)) : nullptr;
    d.trace_cap = prm->trace ? prm->trace_cap : 0;
    h.arena = arena;
    h.arena_bytes = need;
    h.st = d.st;
    h.used = true;
    cudaStream_t st = pool->cur_stream();
    cudaError_t e = cudaMemcpyAsync(dsub, subs.data(), subs.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dball, balls.data(), balls.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dsub1, subs1.data(), subs1.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dbt, bti.data(), bti.size() * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dbl, btl.data(), btl.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { cudaFree(arena); return -(100 + (int)e); }
    pool->slots[s] = h;
    pool->all_dirty = true;
    *s_out = s;
    return COV_OK;
}

// (Re)initialise slot s from `m` codewords exactly as covsearch2e main()
// does (covsearch2e.c:1156-1255): m == M -> rebuild; m < M -> greedy
// placement (or --random-init digits); m > M -> remove-and-repair.
static int slot_init(cov_pool *pool, int s, uint64_t seed, const uint8_t *code, int m, int random_init)
{
    HostSlot &h = pool->slots[s];
    CovSlot &d = h.d;
    const int q = d.q, n = d.n, M = d.M;
    const long long N = d.N;
    if (m < 0 || (m > 0 && !code) || m > h.cap) return COV_EINVAL;
    for (long long i = 0; i < (long long)m * n; i++) if (code[i] >= q) return COV_EINVAL;
    cudaStream_t st = pool->cur_stream();
    if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
    {
        int rc = ensure_attrs();
        if (rc) return rc;
    }
    const bool incremental = m > M || (m < M && !random_init);   // repair or greedy
    if (incremental) CK(cudaMemsetAsync(d.cw, 0, (size_t)N * 4, st));
    CK(cudaMemsetAsync(d.tabu, 0, (size_t)M * n * q * 4, st));
    CK(cudaMemsetAsync(d.P, 0, (size_t)M * (n + 1) * 4, st));
    CK(cudaMemsetAsync(d.ul_bit, 0, (size_t)((N + 31) / 32) * 4, st));
    CovSlotState hs;
    memset(&hs, 0, sizeof hs);
    CovRng rng;
    cov_rng_seed(rng, seed);
    std::vector<uint64_t> pk((size_t)std::max(M, m), 0);
    for (int i = 0; i < m; i++) {
        uint64_t v = 0;
        for (int j = 0; j < n; j++) v |= (uint64_t)code[(size_t)i * n + j] << (4 * j);
        pk[i] = v;
    }
    int have = std::min(m, M);
    const int grid = std::max(1, cov_sm_count()) * 8;
    if (m > M) {
        // remove-and-repair descent (covsearch2e.c:1163-1192): cnt of all m
        // words, then repeatedly drop the first word with the fewest
        // uniquely covered words.
        CovSlot dm = d;
        dm.M = m;
        CK(cudaMemcpyAsync(d.code, pk.data(), (size_t)m * 8, cudaMemcpyHostToDevice, st));
        k_mark_balls<<<grid, 256, 0, st>>>(dm, 0, m, +1);
        CK(cudaGetLastError());
        int *d_u = (int *)d.g_perm;
        std::vector<int> hu(m);
        std::vector<uint64_t> cur(pk.begin(), pk.begin() + m);
        int ms = m;
        while (ms > M) {
            dm.M = ms;
            k_unique_cover<<<ms, 256, 0, st>>>(dm, ms, d_u);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(hu.data(), d_u, sizeof(int) * ms, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            int worst = 0;
            for (int i = 1; i < ms; i++) if (hu[i] < hu[worst]) worst = i;
            k_mark_balls<<<grid, 256, 0, st>>>(dm, worst, 1, -1);
            CK(cudaGetLastError());
            cur.erase(cur.begin() + worst);
            ms--;
            CK(cudaMemcpyAsync(d.code, cur.data(), (size_t)ms * 8, cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
        }
        for (int i = 0; i < M; i++) pk[i] = cur[i];
        have = M;
    }
    unsigned long long *d_z = (unsigned long long *)d.g_dval;
    if (have < M && !random_init) {
        // greedy placement runs on the device (it samples uncovered words)
        CK(cudaMemcpyAsync(d.code, pk.data(), (size_t)M * 8, cudaMemcpyHostToDevice, st));
        if (have > 0) {
            k_mark_balls<<<grid, 256, 0, st>>>(d, 0, have, +1);
            CK(cudaGetLastError());
        }
        CK(cudaMemsetAsync(d_z, 0, 8, st));
        k_count_zero<<<grid, 256, 0, st>>>(d.cw, d.N, d_z);
        CK(cudaGetLastError());
        unsigned long long z = 0;
        CK(cudaMemcpyAsync(&z, d_z, 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < 4; k++) hs.rng[k] = rng.s[k];
        hs.unc = (long long)z;
        hs.best_unc = hs.unc;
        hs.moves_left = have;        // greedy mode: index of the first word to place
        hs.target = -1;
        CK(cudaMemcpyAsync(d.st, &hs, sizeof hs, cudaMemcpyHostToDevice, st));
        int rc = push_slot(pool, s);
        if (rc) return rc;
        std::vector<int> act{s};
        double saved = pool->budget_s;
        pool->budget_s = std::max(saved, 120.0);
        rc = launch_run(pool, act, h.cluster, MODE_GREEDY);
        pool->budget_s = saved;
        if (rc) return rc;
        CK(cudaMemcpyAsync(&hs, d.st, sizeof hs, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hs.status) return hs.status;
        for (int k = 0; k < 4; k++) rng.s[k] = hs.rng[k];
    } else {
        for (int i = have; i < M; i++) {
            uint64_t v = 0;
            for (int j = 0; j < n; j++) v |= (cov_rng_next(rng) % (uint64_t)q) << (4 * j);
            pk[i] = v;
        }
        CK(cudaMemcpyAsync(d.code, pk.data(), (size_t)M * 8, cudaMemcpyHostToDevice, st));
    }
    if (d.fix0) {
        // --fix0 (covsearch2e.c:1241-1253): w -> w - c_0 digit by digit mod q
        // is an isometry, so the code is translated to put codeword 0 at 0^n
        // (the uncovered count does not change) and rebuilt below
        std::vector<uint64_t> cur((size_t)M);
        CK(cudaMemcpyAsync(cur.data(), d.code, (size_t)M * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        const uint64_t c0 = cur[0];
        for (int i = 0; i < M; i++) {
            uint64_t v = 0;
            for (int j = 0; j < n; j++)
                v |= (uint64_t)((cov_nib(cur[i], j) + q - cov_nib(c0, j)) % q) << (4 * j);
            cur[i] = v;
        }
        CK(cudaMemcpyAsync(d.code, cur.data(), (size_t)M * 8, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
    }
    // coverage array, uncovered count, uncovered-word list and private
    // counts of the final M codewords, built tile by tile; then the best code
    CK(cudaMemsetAsync(d_z, 0, 16, st));
    CK(cudaMemsetAsync(d.P, 0, (size_t)M * (n + 1) * 4, st));
    CK(cudaMemsetAsync(d.ul_bit, 0, (size_t)((N + 31) / 32) * 4, st));
    CK(cudaMemsetAsync(d.zb, 0, (size_t)((N + 31) / 32) * 4, st));
    switch (q) {
#define BS_LAUNCH_Q(QQ) \
    case QQ: k_build_state<QQ><<<(unsigned)ipow_h(q, d.bt_nh), BT_NT, bt_smem_bytes(d.bt_tw), st>>>(d, d_z); break;
    BT_Q_LIST(BS_LAUNCH_Q)
#undef BS_LAUNCH_Q
    default: k_build_state<0><<<(unsigned)ipow_h(q, d.bt_nh), BT_NT, bt_smem_bytes(d.bt_tw), st>>>(d, d_z); break;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(d.best, d.code, (size_t)M * 8, cudaMemcpyDeviceToDevice, st));
    unsigned long long zl[2] = {0, 0};
    CK(cudaMemcpyAsync(zl, d_z, 16, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const unsigned long long z = zl[0];
    memset(&hs, 0, sizeof hs);
    for (int k = 0; k < 4; k++) hs.rng[k] = rng.s[k];
    hs.unc = (long long)z;
    hs.best_unc = hs.unc;
    hs.target = -1;
    hs.it_limit = -1;
    hs.sa_T = d.sa_t0;                   // --sa starts at --t0 (covsearch2e.c:1035)
    // the list is in use from the first move when the uncovered words are at
    // most half its capacity -- when the reference's first iteration would
    // rebuild it (covsearch2e.c:1326-1329)
    hs.ul_valid = z <= (unsigned long long)d.ul_cap / 2 && zl[1] == z;
    hs.ul_n = hs.ul_valid ? (int)z : 0;
    hs.finished = hs.unc == 0;
    CK(cudaMemcpyAsync(d.st, &hs, sizeof hs, cudaMemcpyHostToDevice, st));
    int rc = push_slot(pool, s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    return COV_OK;
}

int cov_pool_add(cov_pool *pool, const cov_params *prm, const uint8_t *code, int32_t m,
                 int32_t random_init, int32_t *slot_out)
{
    if (!pool || !prm || (m > 0 && !code) || m < 0) return COV_EINVAL;
    int s = -1;
    int rc = slot_alloc(pool, prm, std::max(m, prm->M), &s);
    if (rc) return rc;
    rc = slot_init(pool, s, prm->seed, code, m, random_init);
    if (rc) {
        cudaFree(pool->slots[s].arena);
        pool->slots[s] = HostSlot();
        pool->all_dirty = true;
        return rc;
    }
    if (slot_out) *slot_out = s;
    return COV_OK;
}

// Re-initialise a live slot with a new seed and code, keeping its storage
// (same q, n, R, M and search parameters).
int cov_pool_load(cov_pool *pool, int32_t slot, uint64_t seed, const uint8_t *code, int32_t m,
                  int32_t random_init)
{
    if (!pool || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    int rc = slot_init(pool, slot, seed, code, m, random_init);
    if (rc) {
        CovSlotState hs;
        memset(&hs, 0, sizeof hs);
        hs.status = rc < 0 && rc > -100 ? rc : COV_ESTATE;
        cudaMemcpy(pool->slots[slot].st, &hs, sizeof hs, cudaMemcpyHostToDevice);
    }
    return rc;
}

// Advance every live instance by up to `moves` further moves (stopping
// early at a full cover or when best <= target).  One launch, one cluster
// per instance; finished instances return at once.  Asynchronous: the work
// is queued on the pool's current stream.
int cov_pool_run_async(cov_pool *pool, int64_t moves, int64_t target)
{
    if (!pool || moves < 0) return COV_EINVAL;
    int rc = refresh_all(pool);
    if (rc) return rc;
    pool->launch_moves = moves;
    return enqueue_step(pool, moves, target);
}

int cov_pool_sync(cov_pool *pool)
{
    if (!pool) return COV_EINVAL;
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return COV_OK;
}

int cov_pool_run(cov_pool *pool, int64_t moves, int64_t target)
{
    int rc = cov_pool_run_async(pool, moves, target);
    if (rc) return rc;
    return cov_pool_sync(pool);
}

// `steps` consecutive runs of `moves` moves captured once as a CUDA graph
// and replayed: one host call per batch of steps.  Asynchronous.
int cov_pool_graph_run(cov_pool *pool, int64_t moves, int64_t target, int32_t steps)
{
    if (!pool || moves < 0 || steps < 1) return COV_EINVAL;
    int rc = refresh_all(pool);
    if (rc) return rc;
    if (pool->n_all == 0) return COV_OK;
    cudaStream_t st = pool->cur_stream();
    if (!pool->gexec || pool->g_moves != moves || pool->g_target != target || pool->g_steps != steps) {
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        pool->launch_moves = moves;
        for (int k = 0; k < steps; k++) {
            rc = enqueue_step(pool, moves, target);
            if (rc) { cudaStreamEndCapture(st, &g); if (g) cudaGraphDestroy(g); return rc; }
        }
        CK(cudaStreamEndCapture(st, &g));
        cudaError_t e = cudaGraphInstantiate(&pool->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { pool->gexec = nullptr; return -(100 + (int)e); }
        pool->g_moves = moves; pool->g_target = target; pool->g_steps = steps;
    }
    CK(cudaGraphLaunch(pool->gexec, st));
    return COV_OK;
}

// Tuning knobs (applied to every slot, present and future):
//   "neg_cluster_pairs"  list x candidate pairs from which the whole cluster
//                        shares the uncovered-list pass (default 4096)
//   "list_cost"          cost of one uncovered-list entry in walked words
//                        (default 5): the entering side reads the list while
//                        U_n * list_cost < ncw (R+1) S', else walks
int cov_pool_set_param(cov_pool *pool, const char *name, int64_t value)
{
    if (!pool || !name) return COV_EINVAL;
    if (!strcmp(name, "grid_help")) {
        // a pool with one slot: share each move's commit with up to `value`
        // helper clusters (0: off)
        if (value < 0 || value > 1024) return COV_EINVAL;
        CK(cudaStreamSynchronize(pool->cur_stream()));
        if (value > 0 && !pool->d_gh) {
            if (cudaMalloc(&pool->d_gh, sizeof(GridHelp)) != cudaSuccess) { cudaGetLastError(); return COV_ENOMEM; }
        }
        pool->grid_help = (int)value;
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    if (!strcmp(name, "grid_help_absent")) {
        // test setting: the helper clusters leave at once, so that the
        // leader's bounded wait for them runs out (status COV_EDRIFT)
        if (value < 0 || value > 1) return COV_EINVAL;
        CK(cudaStreamSynchronize(pool->cur_stream()));
        pool->grid_help_absent = (int)value;
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    if (!strcmp(name, "neg_cluster_pairs")) {
        if (value < 0) return COV_EINVAL;
        pool->neg_cluster_pairs = value;
        for (int s = 0; s < pool->max_slots; s++) {
            if (!pool->slots[s].used) continue;
            pool->slots[s].d.neg_cluster_pairs = value;
            int rc = push_slot(pool, s);
            if (rc) return rc;
        }
        CK(cudaStreamSynchronize(pool->cur_stream()));
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    if (!strcmp(name, "list_cost")) {
        if (value < 0 || value > 1000000) return COV_EINVAL;
        pool->list_cost = (int)value;
        for (int s = 0; s < pool->max_slots; s++) {
            if (!pool->slots[s].used) continue;
            pool->slots[s].d.list_cost = (int)value;
            int rc = push_slot(pool, s);
            if (rc) return rc;
        }
        CK(cudaStreamSynchronize(pool->cur_stream()));
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    return COV_EINVAL;
}

// Free and total device memory of the current device (cudaMemGetInfo): what
// admission of new instances is measured against.
int cov_device_memory(int64_t *free_bytes, int64_t *total_bytes)
{
    if (!free_bytes || !total_bytes) return COV_EINVAL;
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    *free_bytes = (int64_t)f;
    *total_bytes = (int64_t)t;
    return COV_OK;
}

// Per-slot settings:
//   "cluster"            CTAs that advance this slot (1..16); slots of each
//                        cluster size run as one launch, the launches of a
//                        step side by side
//   "neg_cluster_pairs", "list_cost"  as for cov_pool_set_param, this slot only
//   "adjust_mode"        private-count upkeep during a commit: 0 per lane,
//                        1 aggregated per warp, -1 chosen from the expected
//                        number of events (the default)
//   "it_limit"           iteration count at which the slot stops (-1: none);
//                        each run advances it by at most the remainder
//   "wide_sliced"        --wide list pass: 1 finds the hits of up to 64
//                        candidates by bit-sliced counts (the default), 0
//                        tests every candidate against every entry
int cov_pool_set_slot_param(cov_pool *pool, int32_t slot, const char *name, int64_t value)
{
    if (!pool || !name || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    HostSlot &h = pool->slots[slot];
    if (!strcmp(name, "cluster")) {
        if (value < 1 || value > 16) return COV_EINVAL;
        if (h.cluster != (int)value) {
            h.cluster = (int)value;
            pool->all_dirty = true;
        }
        return COV_OK;
    }
    if (!strcmp(name, "neg_cluster_pairs") || !strcmp(name, "list_cost")) {
        if (value < 0 || (name[0] == 'l' && value > 1000000)) return COV_EINVAL;
        if (name[0] == 'n') h.d.neg_cluster_pairs = value;
        else h.d.list_cost = (int)value;
        int rc = push_slot(pool, slot);
        if (rc) return rc;
        CK(cudaStreamSynchronize(pool->cur_stream()));
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    if (!strcmp(name, "adjust_mode") || !strcmp(name, "wide_sliced")) {
        // 0: per-lane private-count updates, 1: warp-aggregated, -1: by estimate
        if (value < (name[0] == 'a' ? -1 : 0) || value > 1) return COV_EINVAL;
        if (name[0] == 'w') h.d.wide_sliced = (int)value;
        else h.d.padj_warp = value < 0 ? padj_auto(h.d.q, h.d.n, h.d.R, h.d.M) : (int)value;
        pool->all_dirty = true;
        int rc = push_slot(pool, slot);
        if (rc) return rc;
        CK(cudaStreamSynchronize(pool->cur_stream()));
        if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
        return COV_OK;
    }
    if (!strcmp(name, "it_limit")) {
        if (value < -1) return COV_EINVAL;
        long long v = value;
        CK(cudaMemcpyAsync(&h.st->it_limit, &v, sizeof v, cudaMemcpyHostToDevice, pool->cur_stream()));
        CK(cudaStreamSynchronize(pool->cur_stream()));
        return COV_OK;
    }
    return COV_EINVAL;
}

// Run on the caller's stream (a cudaStream_t passed as void*); NULL returns
// to the pool's own stream.
int cov_pool_set_stream(cov_pool *pool, void *stream)
{
    if (!pool) return COV_EINVAL;
    CK(cudaStreamSynchronize(pool->cur_stream()));
    pool->ext = (cudaStream_t)stream;
    pool->use_ext = stream != nullptr;
    if (pool->gexec) { cudaGraphExecDestroy(pool->gexec); pool->gexec = nullptr; }
    return COV_OK;
}

// statuses of slots 0..n-1 in one device-to-host copy (unused slots: status
// COV_ESTATE)
int cov_pool_status_all(cov_pool *pool, cov_status *out, int32_t n)
{
    if (!pool || !out || n < 0 || n > pool->max_slots) return COV_EINVAL;
    std::vector<CovSlotState> hs(pool->max_slots);
    CK(cudaMemcpyAsync(hs.data(), pool->d_states, sizeof(CovSlotState) * pool->max_slots,
                       cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    for (int s = 0; s < n; s++) {
        cov_status &o = out[s];
        memset(&o, 0, sizeof o);
        if (!pool->slots[s].used) { o.status = COV_ESTATE; continue; }
        const CovSlotState &h = hs[s];
        o.it = h.it; o.uncovered = h.unc; o.best = h.best_unc; o.kicks = h.nkicks;
        o.status = h.status; o.finished = h.unc <= 0; o.ul_valid = h.ul_valid; o.ul_n = h.ul_n;
        o.trace_n = h.trace_n;
    }
    return COV_OK;
}

int cov_pool_status(cov_pool *pool, int32_t slot, cov_status *out)
{
    if (!pool || !out || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    CovSlotState hs;
    int rc = read_state(pool, slot, &hs);
    if (rc) return rc;
    memset(out, 0, sizeof *out);
    out->it = hs.it;
    out->uncovered = hs.unc;
    out->best = hs.best_unc;
    out->kicks = hs.nkicks;
    out->status = hs.status;
    out->finished = hs.unc <= 0;
    out->ul_valid = hs.ul_valid;
    out->ul_n = hs.ul_n;
    out->trace_n = hs.trace_n;
    return COV_OK;
}

static int get_packed(cov_pool *pool, int32_t slot, bool best, uint8_t *out)
{
    if (!pool || !out || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    const CovSlot &d = pool->slots[slot].d;
    std::vector<uint64_t> pk(d.M);
    CK(cudaMemcpyAsync(pk.data(), best ? d.best : d.code, (size_t)d.M * 8, cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    for (int i = 0; i < d.M; i++)
        for (int j = 0; j < d.n; j++) out[(size_t)i * d.n + j] = (uint8_t)cov_nib(pk[i], j);
    return COV_OK;
}

int cov_pool_get_code(cov_pool *pool, int32_t slot, uint8_t *out) { return get_packed(pool, slot, false, out); }
int cov_pool_get_best(cov_pool *pool, int32_t slot, uint8_t *out) { return get_packed(pool, slot, true, out); }

int cov_pool_get_cnt(cov_pool *pool, int32_t slot, uint16_t *out)
{
    if (!pool || !out || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    const CovSlot &d = pool->slots[slot].d;
    uint16_t *tmp = nullptr;
    CK(cudaMallocAsync(&tmp, (size_t)d.N * 2, pool->cur_stream()));
    k_unpack_cnt<<<std::max(1, cov_sm_count()) * 4, 256, 0, pool->cur_stream()>>>(d.cw, d.N, tmp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, tmp, (size_t)d.N * 2, cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaFreeAsync(tmp, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return COV_OK;
}

int cov_pool_get_private(cov_pool *pool, int32_t slot, int32_t *out)
{
    if (!pool || !out || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    const CovSlot &d = pool->slots[slot].d;
    CK(cudaMemcpyAsync(out, d.P, (size_t)d.M * (d.n + 1) * 4, cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return COV_OK;
}

int cov_pool_get_trace(cov_pool *pool, int32_t slot, cov_move_rec *out, int64_t cap, int64_t *n_out)
{
    if (!pool || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    const CovSlot &d = pool->slots[slot].d;
    CovSlotState hs;
    int rc = read_state(pool, slot, &hs);
    if (rc) return rc;
    long long n = std::min<long long>(hs.trace_n, d.trace_cap);
    if (out && cap > 0) {
        long long k = std::min<long long>(n, cap);
        if (k > 0)
            CK(cudaMemcpyAsync(out, d.trace, (size_t)k * sizeof(cov_move_rec), cudaMemcpyDeviceToHost, pool->cur_stream()));
        CK(cudaStreamSynchronize(pool->cur_stream()));
    }
    if (n_out) *n_out = n;
    return COV_OK;
}

int cov_pool_get_rng(cov_pool *pool, int32_t slot, uint64_t *out4)
{
    if (!pool || !out4 || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    CovSlotState hs;
    int rc = read_state(pool, slot, &hs);
    if (rc) return rc;
    for (int k = 0; k < 4; k++) out4[k] = hs.rng[k];
    return COV_OK;
}

// leader phase cycle counts (24) followed by the list-pair counter
int cov_pool_get_prof(cov_pool *pool, int32_t slot, uint64_t *out25)
{
    if (!pool || !out25 || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    CovSlotState hs;
    int rc = read_state(pool, slot, &hs);
    if (rc) return rc;
    for (int k = 0; k < 24; k++) out25[k] = hs.prof[k];
    out25[24] = (uint64_t)hs.stat_ul_pairs;
    return COV_OK;
}

int cov_pool_get_tabu(cov_pool *pool, int32_t slot, int32_t *out)
{
    if (!pool || !out || slot < 0 || slot >= pool->max_slots || !pool->slots[slot].used) return COV_EINVAL;
    const CovSlot &d = pool->slots[slot].d;
    CK(cudaMemcpyAsync(out, d.tabu, (size_t)d.M * d.n * d.q * 4, cudaMemcpyDeviceToHost, pool->cur_stream()));
    CK(cudaStreamSynchronize(pool->cur_stream()));
    return COV_OK;
}

}  // extern "C"
