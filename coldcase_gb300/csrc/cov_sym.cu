// cov_sym.cu -- GB300 (sm_103a) quotient search for covering codes that are
// invariant under the diagonal translation x -> x + 1^n:
// cov/engine/symsearch.c on the GPU.
//
// The code is a union of orbits {(j, e + j) : j in Z_q}; an orbit covers the
// quotient word d in Z_q^(n-1) once per centre e + delta within radius
// R - [delta != 0] (symsearch.c:15-31), so the whole search runs on q^(n-1)
// counters.  The trajectory is the reference's, move for move: the RNG
// stream, the 64 probes then cyclic scan of the pick, the candidate order
// (orbit, delta, position), the Fisher-Yates sample, the read-only estimate
// of every sampled move (each of its q sub-moves judged against the
// unchanged counters), the reservoir tie-break and the kicks.
//
// Execution: one thread-block cluster per instance.  The leader CTA does the
// serial, RNG-ordered steps (pick, candidates, sample, selection); the
// cluster shares the three bulk operations -- the estimates of all sampled
// moves (take x S' counter pairs, S' = C(n-1,R)(q-1)^R), the commit of the
// chosen move (S' pairs) and the q balls of an orbit (init and kicks).  Ops
// go out through the leader's shared memory and CTAs meet only at hardware
// cluster barriers.  Counters are 16 bits (as the reference's), two to a
// 32-bit word, updated by 32-bit atomics: a count never exceeds 65000 and
// never drops below zero, so one half never carries into the other.  Beside
// them a 2-bit shadow min(cnt, 2) (4 words a byte, the layout of
// covsearch2e's opt_st = 2) serves the estimates and the pick: 8 MB for the
// 16.7M quotient words of K_8(9,4), so that many instances stay in L2.
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cooperative_groups.h>
#include "cov_common.cuh"
#include "../../include/covgpu.h"

namespace cg = cooperative_groups;

#define SNT 512                 // threads per CTA
#define SNW (SNT / 32)
#define SYM_TS 4096             // candidates held in shared memory
#define SYM_MAXR 7              // symsearch.c:311
#define SYM_PB 16               // pick probes drawn per batch
#define SYM_CT 2048             // centre-table entries (sampled candidates x q)
#define SYM_INV 2048            // moduli with a reciprocal in shared memory
#define SYM_CYCLES_PER_NS 2ull

enum { SOP_STOP = 0, SOP_ORBIT = 1, SOP_EVAL = 2, SOP_COMMIT = 3 };
enum { SPH_INIT = 0, SPH_MOVE = 1, SPH_SELECT = 2, SPH_AFTER_COMMIT = 3, SPH_KICK_DEL = 4,
       SPH_KICK_ADD = 5, SPH_KICK_NEXT = 6, SPH_DONE = 7, SPH_EVAL = 8 };
enum { SMODE_INIT = 0, SMODE_RUN = 1 };

struct SymState {
    uint64_t rng[4];
    long long it, unc, best_unc, since_improve, nkicks, trace_n, moves_left, it_limit;
    int init_i;                  // orbits placed by the greedy initialisation
    int status, finished, pad;
    // leader cycles by phase, accumulated over launches: 0 pick, 1
    // candidates, 2 sample, 3 estimate op, 4 selection, 5 commit op, 6 orbit
    // ops, 7 the rest; 8 moves counted
    unsigned long long prof[9];
    // a move planned up to its estimates, which a grid-wide launch computes
    // (the sample is in cands[0..take)); the next leader launch goes on
    // from the selection
    int eval_pending, take;
    cov_move_rec rec;
};

struct SymSlot {
    int q, n, R, NR, norb;
    uint32_t N;                  // q^(n-1)
    uint32_t pw[COV_MAXN];       // q^(NR-1-j)
    uint32_t ppow[COV_MAXN + 1]; // (q-1)^k
    int kick, cand;
    long long stall;
    int rs;                      // max(R,1): row stride of the subset tables
    int wnc[2];                  // C(NR-1,R), C(NR-1,R-1): subsets of a sub-move walk
    uint32_t witems[2];          // walk items of a sub-move of radius R / R-1
    uint32_t ipc;                // walk items of one candidate (its q sub-moves)
    uint32_t bcum[SYM_MAXR + 2]; // ball items of radius 1..r-1 (centre excluded)
    uint32_t bitems[2];          // ball items of radius R / R-1 (centre included)
    uint32_t opi;                // ball items of one orbit
    int boff[SYM_MAXR + 2];      // first r-subset of bsub
    const uint8_t *wsub[2];      // [NR][wnc][rs]: subsets avoiding position p
    const uint8_t *bsub;         // r-subsets of all NR positions, r = 1..R
    uint32_t inv_qm1;            // ceil(2^32 / (q-1))
    uint64_t inv_pp[SYM_MAXR + 1];   // ceil(2^64 / (q-1)^k)
    uint64_t inv_wit1, inv_bit1;     // ceil(2^64 / witems[1]), ceil(2^64 / bitems[1])
    uint64_t inv_ipc;                // ceil(2^64 / ipc)
    uint64_t inv_N;                  // floor((2^64-1) / N)
    uint32_t *cnt2;              // [ceil(N/2)] two 16-bit counters per word
    uint32_t *st2;               // min(cnt, 2) per word, 2 bits each; padded to whole
                                 // 16-byte windows plus one
    uint64_t *rep, *best;        // [norb] representatives, packed digits
    uint32_t *cands;             // [norb*q*NR + 8] candidates (oversized case)
    int32_t *cd;                 // [norb*q*NR + 8] estimates
    cov_move_rec *trace;
    long long trace_cap;
    SymState *st;
};

// centres of one orbit's q balls and, for a move, their word offsets
struct SymCentres {
    uint64_t cpk[COV_MAXQ];
    uint32_t base[COV_MAXQ];
    uint32_t dv[COV_MAXQ];
};

struct SymSmem {
    SymSlot slot;
    SymCentres ct;
    // op broadcast by the leader (read by every CTA through DSMEM)
    int op, oi, opos, oval, osign, take;
    unsigned long long acc;      // uncovered change accumulated by an op
    // leader state
    CovRng rng;
    long long it, unc, best_unc, since_improve, nkicks, trace_n, moves_left, it_limit;
    int init_i, status, finished, phase, kick_t, cand_sm;
    int split, eval_pending;     // estimates by a grid-wide launch; one is due
    unsigned long long deadline;
    long long guard, est;
    unsigned long long prof[9];
    long long t_mark;
    cov_move_rec rec;
    // scratch
    int red_i[SNW];
    long long red_ll[SNW];
    int ibc[4];
    uint32_t probe[SYM_PB];
    CovRng pstate[SYM_PB];
    uint32_t cand[SYM_TS];       // candidates (leader); the sample (every CTA)
    uint64_t tcpk[SYM_CT];       // centres of the sampled candidates: [s*q + delta]
    uint32_t tbase[SYM_CT];
    uint32_t tdv[SYM_CT];
    uint64_t inv[SYM_INV + 1];   // floor((2^64-1)/m): leader's modular reductions
    int32_t cdv[SYM_TS];
    uint8_t skip[SYM_TS];
};

// ------------------------------------------------------------ helpers ----
__device__ __forceinline__ int sym_cnt(const SymSlot &d, uint32_t w)
{
    return (int)cov_ldcg(reinterpret_cast<const unsigned short *>(d.cnt2) + w);
}

// add s = +1 / -1 to counter w; returns the count before
__device__ __forceinline__ int sym_add(const SymSlot &d, uint32_t w, int s)
{
    const uint32_t sh = (w & 1u) * 16u;
    const uint32_t old = atomicAdd(&d.cnt2[w >> 1], (uint32_t)s << sh);
    return (int)((old >> sh) & 0xffffu);
}

// min(cnt[w], 2) from the shadow
__device__ __forceinline__ int sym_st(const SymSlot &d, uint32_t w)
{
    return (int)((cov_ldcg(&d.st2[w >> 4]) >> (2u * (w & 15u))) & 3u);
}

// bring the shadow of w in line with its (final) count
__device__ __forceinline__ void sym_fix(const SymSlot &d, uint32_t w)
{
    const int c = min(sym_cnt(d, w), 2);
    const uint32_t sh = 2u * (w & 15u);
    uint32_t *word = &d.st2[w >> 4];
    if ((int)((cov_ldcg(word) >> sh) & 3u) == c) return;
    atomicAnd(word, ~(3u << sh));
    if (c) atomicOr(word, (uint32_t)c << sh);
}

__device__ __forceinline__ void sym_error(const SymSlot &d, int code)
{
    atomicCAS(&d.st->status, 0, code);
}

__device__ __forceinline__ long long sym_clock()
{
    long long t;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t) :: "memory");
    return t;
}

__device__ __forceinline__ void sym_bar()
{
    __syncwarp();
    __syncthreads();
}

__device__ long long sym_block_sum(SymSmem &S, long long v)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5;
    sym_bar();
    if ((threadIdx.x & 31) == 0) S.red_ll[w] = v;
    sym_bar();
    long long t = 0;
    for (int k = 0; k < SNW; k++) t += S.red_ll[k];
    sym_bar();
    return t;
}

__device__ int sym_block_min(SymSmem &S, int v)
{
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5;
    sym_bar();
    if ((threadIdx.x & 31) == 0) S.red_i[w] = v;
    sym_bar();
    int t = 0x7fffffff;
    for (int k = 0; k < SNW; k++) t = min(t, S.red_i[k]);
    sym_bar();
    return t;
}

// exclusive prefix of v over the block; *total gets the sum
__device__ int sym_block_scan(SymSmem &S, int v, int *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    sym_bar();
    if (lane == 31) S.red_i[w] = x;
    sym_bar();
    int before = 0, tot = 0;
    for (int k = 0; k < SNW; k++) {
        if (k < w) before += S.red_i[k];
        tot += S.red_i[k];
    }
    sym_bar();
    *total = tot;
    return before + x - v;
}

// digit j of the centre e + delta
__device__ __forceinline__ int sym_cdig(const SymSlot &d, uint64_t e, int delta, int j)
{
    int c = cov_nib(e, j) + delta;
    return c >= d.q ? c - d.q : c;
}

__device__ __forceinline__ uint32_t sym_centre(const SymSlot &d, uint64_t e, int delta)
{
    uint32_t x = 0;
    for (int j = 0; j < d.NR; j++) x += (uint32_t)sym_cdig(d, e, delta, j) * d.pw[j];
    return x;
}

// ----------------------------------------------------------- the walks ----
// Divisions by the slot's fixed divisors go through multiply-high with
// precomputed reciprocals: x / (q-1) for x < 2^24 with a 32-bit one, x / m
// for x < 2^32 with a 64-bit one (both exact in those ranges).
__device__ __forceinline__ uint32_t sym_div_qm1(const SymSlot &d, uint32_t x)
{
    return d.q == 2 ? x : __umulhi(x, d.inv_qm1);
}
__device__ __forceinline__ uint32_t sym_div64(uint32_t x, uint32_t m, uint64_t inv)
{
    return m == 1 ? x : (uint32_t)__umul64hi((uint64_t)x, inv);
}

// Centres of the q balls of orbit e (radius R at e, R-1 at e + delta) and,
// for a move of position p to v, the offset each centre's word index moves
// by (symsearch.c:162-174, :216-224); built by threads 0..q-1.
__device__ void sym_centres(const SymSlot &d, SymCentres &C, uint64_t e, int p, int v)
{
    const int dl = threadIdx.x;
    if (dl < d.q && d.R - (dl != 0) >= 0) {
        uint64_t c = 0;
        uint32_t x = 0;
        for (int j = 0; j < d.NR; j++) {
            int cj = cov_nib(e, j) + dl;
            if (cj >= d.q) cj -= d.q;
            c = cov_setnib(c, j, cj);
            x += (uint32_t)cj * d.pw[j];
        }
        C.cpk[dl] = c;
        C.base[dl] = x;
        if (p >= 0) {
            int nv = v + dl;
            if (nv >= d.q) nv -= d.q;
            C.dv[dl] = (uint32_t)((nv - cov_nib(c, p)) * (int)d.pw[p]);
        }
    }
}

// one 32-bit word of the eight loaded as two uint4
__device__ __forceinline__ uint32_t sym_pick8(const uint4 &lo, const uint4 &hi, int i)
{
    const uint4 &h = (i & 4) ? hi : lo;
    return (i & 2) ? ((i & 1) ? h.w : h.z) : ((i & 1) ? h.y : h.x);
}

// Walk item r in [0, ipc) of a move of position p: its sub-move delta, one
// subset of the other positions and values for all but the subset's last
// position; the q-1 values of the last position are the inner loop.  Each
// word a differs from the centre exactly on the subset; b is a with
// position p moved (symsearch.c:177-205).  MODE 0: (cnt[a]==1) - (cnt[b]==0)
// against the unchanged counters (read from the 2-bit shadow); MODE 1: the
// move itself on the counters; MODE 2: refresh the shadow of a and b.
// cpk/base/dv: the centres' packed digits, word indices and move offsets,
// indexed by delta.
template <int MODE>
__device__ __forceinline__ long long sym_walk_item(const SymSlot &d, const uint64_t *cpk, const uint32_t *cbase,
                                                   const uint32_t *cdv, int p, uint32_t r)
{
    int delta = 0;
    uint32_t loc = r;
    if (r >= d.witems[0]) {
        const uint32_t k = sym_div64(r - d.witems[0], d.witems[1], d.inv_wit1);
        delta = 1 + (int)k;
        loc = r - d.witems[0] - k * d.witems[1];
    }
    const int t = delta ? 1 : 0, rad = d.R - t;
    const uint64_t c = cpk[delta];
    const uint32_t base = cbase[delta], dv = cdv[delta];
    long long du = 0;
    auto visit = [&](uint32_t a) {
        const uint32_t b = a + dv;
        if (MODE == 1) {
            const int oa = sym_add(d, a, -1);
            if (oa == 0) sym_error(d, COV_EDRIFT);
            du += oa == 1;
            du -= sym_add(d, b, +1) == 0;
        } else if (MODE == 2) {
            sym_fix(d, a);
            sym_fix(d, b);
        }
    };
    if (rad == 0) {
        if (MODE == 0) du += (long long)(sym_st(d, base) == 1) - (long long)(sym_st(d, base + dv) == 0);
        else visit(base);
        return du;
    }
    const uint32_t pp = d.ppow[rad - 1];
    const uint32_t kk = sym_div64(loc, pp, d.inv_pp[rad - 1]);
    uint32_t rem = loc - kk * pp;
    const uint8_t *ps = d.wsub[t] + ((size_t)p * d.wnc[t] + kk) * d.rs;
    const int qm1 = d.q - 1;
    uint32_t w = base;
    for (int k = rad - 2; k >= 0; --k) {
        const uint32_t qt = sym_div_qm1(d, rem);
        const int dig = (int)(rem - qt * (uint32_t)qm1);
        rem = qt;
        const int j = ps[k], cj = cov_nib(c, j);
        w += (uint32_t)((dig + (dig >= cj) - cj) * (int)d.pw[j]);
    }
    const int last = ps[rad - 1], cl = cov_nib(c, last);
    const int pl = (int)d.pw[last];
    if constexpr (MODE == 0) {
        const uint32_t a0 = w - (uint32_t)(cl * pl);       // the word with digit 0 at `last`
        if (d.q * pl <= 64) {
            // the q words a0 + v pl lie in two aligned 16-byte windows of the
            // shadow (64 words each); so do the b words
            auto count = [&](uint32_t x0, int want) -> int {
                const uint32_t w0 = x0 & ~63u;
                const uint4 lo = __ldcg(reinterpret_cast<const uint4 *>(d.st2 + (w0 >> 4)));
                uint4 hi = make_uint4(0, 0, 0, 0);
                if (x0 + (uint32_t)(qm1 * pl) >= w0 + 64) hi = __ldcg(reinterpret_cast<const uint4 *>(d.st2 + (w0 >> 4) + 4));
                if (pl == 1) {
                    // q consecutive 2-bit fields: compare all at once
                    const int off = (int)(x0 - w0), wi = off >> 4;
                    const uint32_t ch = __funnelshift_r(sym_pick8(lo, hi, wi), sym_pick8(lo, hi, wi + 1),
                                                        2 * (off & 15));
                    const uint32_t fm = (d.q == 16 ? 0xffffffffu : ((1u << (2 * d.q)) - 1u)) & 0x55555555u &
                                        ~(1u << (2 * cl));
                    const uint32_t b0 = ch & fm, b1 = (ch >> 1) & fm;
                    return __popc(want ? (b0 & ~b1) : (fm & ~b0 & ~b1));
                }
                int n = 0;
                for (int v = 0; v <= qm1; v++) {
                    if (v == cl) continue;
                    const int x = (int)(x0 - w0) + v * pl;
                    n += (int)((sym_pick8(lo, hi, x >> 4) >> (2 * (x & 15))) & 3u) == want;
                }
                return n;
            };
            return (long long)count(a0, 1) - (long long)count(a0 + dv, 0);
        }
        // otherwise all 2(q-1) reads of the item are issued before any is used
        int ca[COV_MAXQ - 1], cb[COV_MAXQ - 1];
#pragma unroll
        for (int k = 0; k < COV_MAXQ - 1; k++) {
            if (k < qm1) {
                const uint32_t a = w + (uint32_t)((k + (k >= cl) - cl) * pl);
                ca[k] = sym_st(d, a);
                cb[k] = sym_st(d, a + dv);
            }
        }
#pragma unroll
        for (int k = 0; k < COV_MAXQ - 1; k++)
            if (k < qm1) du += (long long)(ca[k] == 1) - (long long)(cb[k] == 0);
        return du;
    } else {
        for (int k = 0; k < qm1; k++) visit(w + (uint32_t)((k + (k >= cl) - cl) * pl));
        return du;
    }
}

// Ball item r in [0, opi) of an orbit (centres in C): +1 / -1 on every word
// it names (MODE 1, symsearch.c:135-174; returns the uncovered change) or
// the refresh of their shadow (MODE 2)
template <int MODE>
__device__ __forceinline__ long long sym_ball_item(const SymSlot &d, const SymCentres &C, uint32_t r, int sign)
{
    int delta = 0;
    uint32_t loc = r;
    if (r >= d.bitems[0]) {
        const uint32_t k = sym_div64(r - d.bitems[0], d.bitems[1], d.inv_bit1);
        delta = 1 + (int)k;
        loc = r - d.bitems[0] - k * d.bitems[1];
    }
    const int qm1 = d.q - 1;
    const uint64_t c = C.cpk[delta];
    const uint32_t base = C.base[delta];
    long long du = 0;
    auto touch = [&](uint32_t w) {
        if (MODE == 2) { sym_fix(d, w); return; }
        const int old = sym_add(d, w, sign);
        if (sign > 0) du -= old == 0;
        else {
            if (old == 0) sym_error(d, COV_EDRIFT);
            du += old == 1;
        }
    };
    if (loc == 0) { touch(base); return du; }
    loc -= 1;
    int rr = 1;
    while (rr <= SYM_MAXR && loc >= d.bcum[rr + 1]) rr++;
    loc -= d.bcum[rr];
    const uint32_t pp = d.ppow[rr - 1];
    const uint32_t kk = sym_div64(loc, pp, d.inv_pp[rr - 1]);
    uint32_t rem = loc - kk * pp;
    const uint8_t *ps = d.bsub + (size_t)(d.boff[rr] + (int)kk) * d.rs;
    uint32_t w = base;
    for (int k = rr - 2; k >= 0; --k) {
        const uint32_t qt = sym_div_qm1(d, rem);
        const int dig = (int)(rem - qt * (uint32_t)qm1);
        rem = qt;
        const int j = ps[k], cj = cov_nib(c, j);
        w += (uint32_t)((dig + (dig >= cj) - cj) * (int)d.pw[j]);
    }
    const int last = ps[rr - 1], cl = cov_nib(c, last);
    const int pl = (int)d.pw[last];
    for (int k = 0; k < qm1; k++) touch(w + (uint32_t)((k + (k >= cl) - cl) * pl));
    return du;
}

// ----------------------------------------------------------------- ops ----
// The counters change first; after a cluster barrier the same words get
// their shadow refreshed from the final counts (a word may be touched by
// several threads, so the shadow is only written once its count is final).
__device__ void sym_op_orbit(const SymSlot &d, SymSmem &S, SymSmem *LS, cg::cluster_group &cl, int rank,
                             int csize, int i, int sign)
{
    sym_centres(d, S.ct, cov_ldcg(&d.rep[i]), -1, 0);
    sym_bar();
    long long du = 0;
    const uint32_t stride = (uint32_t)csize * SNT;
    for (uint32_t r = (uint32_t)rank * SNT + threadIdx.x; r < d.opi; r += stride)
        du += sym_ball_item<1>(d, S.ct, r, sign);
    du = sym_block_sum(S, du);
    if (threadIdx.x == 0 && du) atomicAdd(&LS->acc, (unsigned long long)du);
    cl.sync();
    for (uint32_t r = (uint32_t)rank * SNT + threadIdx.x; r < d.opi; r += stride) sym_ball_item<2>(d, S.ct, r, 0);
}

// Estimates of the sampled moves.  Flat: every CTA holds the centres of all
// sampled candidates (take x q entries) and the cluster's threads run over
// all (candidate, item) pairs at once.  Nested, for samples too large for
// that table: candidate by candidate, the threads splitting its items.
// (S.cand holds the sample when take <= SYM_TS; `rank` of `csize` CTAs;
// GRID: the whole grid runs it, else one cluster)
template <bool GRID>
__device__ void sym_eval_items(const SymSlot &d, SymSmem &S, int rank, int csize, int take)
{
    const bool sm = take <= SYM_TS;
    const uint32_t stride = (uint32_t)csize * SNT;
    const int q = d.q;
    if (sm && take * q <= SYM_CT && (unsigned long long)take * d.ipc < (1ull << 32)) {
        for (int x = threadIdx.x; x < take * q; x += SNT) {
            const int s = x / q, dl = x - s * q;
            if (d.R - (dl != 0) < 0) continue;
            const uint32_t c = S.cand[s];
            const uint64_t e = cov_ldcg(&d.rep[c >> 8]);
            const int p = (int)((c >> 4) & 15u), v = (int)(c & 15u);
            uint64_t pk = 0;
            uint32_t xw = 0;
            for (int j = 0; j < d.NR; j++) {
                int cj = cov_nib(e, j) + dl;
                if (cj >= q) cj -= q;
                pk = cov_setnib(pk, j, cj);
                xw += (uint32_t)cj * d.pw[j];
            }
            int nv = v + dl;
            if (nv >= q) nv -= q;
            S.tcpk[x] = pk;
            S.tbase[x] = xw;
            S.tdv[x] = (uint32_t)((nv - cov_nib(pk, p)) * (int)d.pw[p]);
        }
        sym_bar();
        const uint32_t total = (uint32_t)take * d.ipc;
        if (!GRID) {
            // one cluster: items strided over its threads
            int cur = -1, p = 0;
            long long acc = 0;
            for (uint32_t t = (uint32_t)rank * SNT + threadIdx.x; t < total; t += stride) {
                const int s2 = (int)sym_div64(t, d.ipc, d.inv_ipc);
                const uint32_t r = t - (uint32_t)s2 * d.ipc;
                if (s2 != cur) {
                    if (cur >= 0 && acc) atomicAdd(&d.cd[cur], (int)acc);
                    cur = s2;
                    acc = 0;
                    p = (int)((S.cand[s2] >> 4) & 15u);
                }
                const int o = s2 * q;
                acc += sym_walk_item<0>(d, S.tcpk + o, S.tbase + o, S.tdv + o, p, r);
            }
            if (cur >= 0 && acc) atomicAdd(&d.cd[cur], (int)acc);
            return;
        }
        // the whole grid: each warp takes a contiguous run of items, 32 at a
        // time, so that a lane's sum stays on one candidate for long
        // stretches (strided items would send an atomic per item to a few
        // dozen estimates); sums reach the estimates when the candidate
        // changes and, warp-reduced, at the end of the run
        const int lane = threadIdx.x & 31;
        const uint32_t nwarps = (uint32_t)csize * SNW;
        const uint32_t gw = (uint32_t)rank * SNW + (threadIdx.x >> 5);
        const uint32_t seg = ((total + nwarps - 1) / nwarps + 31u) & ~31u;
        const uint32_t lo = (uint32_t)min((unsigned long long)total, (unsigned long long)gw * seg);
        const uint32_t hi = (uint32_t)min((unsigned long long)total, (unsigned long long)lo + seg);
        int cur = -1, p = 0;
        long long acc = 0;
        for (uint32_t t0 = lo; t0 < hi; t0 += 32) {
            const uint32_t t = t0 + (uint32_t)lane;
            if (t < hi) {
                const int s2 = (int)sym_div64(t, d.ipc, d.inv_ipc);
                const uint32_t r = t - (uint32_t)s2 * d.ipc;
                if (s2 != cur) {
                    if (cur >= 0 && acc) atomicAdd(&d.cd[cur], (int)acc);
                    cur = s2;
                    acc = 0;
                    p = (int)((S.cand[s2] >> 4) & 15u);
                }
                const int o = s2 * q;
                acc += sym_walk_item<0>(d, S.tcpk + o, S.tbase + o, S.tdv + o, p, r);
            }
        }
        const int c0 = __shfl_sync(0xffffffffu, cur, 0);
        if (__all_sync(0xffffffffu, cur == c0)) {
            for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0 && c0 >= 0 && acc) atomicAdd(&d.cd[c0], (int)acc);
        } else if (cur >= 0 && acc) {
            atomicAdd(&d.cd[cur], (int)acc);
        }
        return;
    }
    for (int s = 0; s < take; s++) {
        const uint32_t c = sm ? S.cand[s] : cov_ldcg(&d.cands[s]);
        const int p = (int)((c >> 4) & 15u), v = (int)(c & 15u);
        sym_centres(d, S.ct, cov_ldcg(&d.rep[c >> 8]), p, v);
        sym_bar();
        long long acc = 0;
        for (uint32_t r = (uint32_t)rank * SNT + threadIdx.x; r < d.ipc; r += stride)
            acc += sym_walk_item<0>(d, S.ct.cpk, S.ct.base, S.ct.dv, p, r);
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&d.cd[s], (int)acc);
        sym_bar();
    }
}

__device__ void sym_op_commit(const SymSlot &d, SymSmem &S, SymSmem *LS, cg::cluster_group &cl, int rank,
                              int csize, int i, int p, int v)
{
    sym_centres(d, S.ct, cov_ldcg(&d.rep[i]), p, v);
    sym_bar();
    long long du = 0;
    const uint32_t stride = (uint32_t)csize * SNT;
    for (uint32_t r = (uint32_t)rank * SNT + threadIdx.x; r < d.ipc; r += stride)
        du += sym_walk_item<1>(d, S.ct.cpk, S.ct.base, S.ct.dv, p, r);
    du = sym_block_sum(S, du);
    if (threadIdx.x == 0 && du) atomicAdd(&LS->acc, (unsigned long long)du);
    cl.sync();
    for (uint32_t r = (uint32_t)rank * SNT + threadIdx.x; r < d.ipc; r += stride)
        sym_walk_item<2>(d, S.ct.cpk, S.ct.base, S.ct.dv, p, r);
}

__device__ void sym_op_eval(const SymSlot &d, SymSmem &S, SymSmem *LS, int rank, int csize, int take)
{
    if (take <= SYM_TS && rank != 0) {
        for (int s = threadIdx.x; s < take; s += SNT) S.cand[s] = LS->cand[s];
        sym_bar();
    }
    sym_eval_items<false>(d, S, rank, csize, take);
}

// ------------------------------------------------------ leader routines ----
__device__ __forceinline__ uint64_t sym_draw(SymSmem &S) { return cov_rng_next(S.rng); }

// x mod m through a reciprocal (one correction at most): the table for small
// m, the slot's own for N
__device__ __forceinline__ uint64_t sym_mod(const SymSmem &S, uint64_t x, uint64_t m)
{
    if (m <= SYM_INV) {
        const uint64_t qe = __umul64hi(x, S.inv[m]);
        uint64_t r = x - qe * m;
        while (r >= m) r -= m;
        return r;
    }
    return x % m;
}
__device__ __forceinline__ uint32_t sym_modN(const SymSlot &d, uint64_t x)
{
    const uint64_t qe = __umul64hi(x, d.inv_N);
    uint64_t r = x - qe * (uint64_t)d.N;
    while (r >= (uint64_t)d.N) r -= (uint64_t)d.N;
    return (uint32_t)r;
}

// 64 uniform probes, then the first zero cyclically after a random start
// (symsearch.c:268-280).  Probes are drawn in batches with the generator
// state after each draw, so that exactly the draws the reference makes are
// consumed.
__device__ long long sym_pick(const SymSlot &d, SymSmem &S)
{
    const int tid = threadIdx.x;
    for (int b0 = 0; b0 < 64; b0 += SYM_PB) {
        if (tid == 0) {
            CovRng r = S.rng;
            for (int k = 0; k < SYM_PB; k++) {
                S.probe[k] = sym_modN(d, cov_rng_next(r));
                S.pstate[k] = r;
            }
        }
        sym_bar();
        int hit = 0x7fffffff;
        if (tid < SYM_PB && sym_st(d, S.probe[tid]) == 0) hit = tid;
        hit = sym_block_min(S, hit);
        if (hit != 0x7fffffff) {
            const long long w = S.probe[hit];
            sym_bar();
            if (tid == 0) S.rng = S.pstate[hit];
            sym_bar();
            return w;
        }
        if (tid == 0) S.rng = S.pstate[SYM_PB - 1];
        sym_bar();
    }
    if (tid == 0) S.ibc[0] = (int)sym_modN(d, sym_draw(S));
    sym_bar();
    const uint32_t start = (uint32_t)S.ibc[0];
    sym_bar();
    for (uint32_t off = 0; off < d.N; off += SNT * 4) {
        int best = 0x7fffffff;
        for (int k = 0; k < 4; k++) {
            const uint32_t o = off + (uint32_t)k * SNT + (uint32_t)tid;
            if (o >= d.N) break;
            // (start + o) may pass 2^32 when the quotient has over 2^31 words
            unsigned long long w = (unsigned long long)start + o;
            if (w >= d.N) w -= d.N;
            if (sym_st(d, (uint32_t)w) == 0) { best = (int)(o - off); break; }
        }
        best = sym_block_min(S, best);
        if (best != 0x7fffffff) {
            unsigned long long w = (unsigned long long)start + off + (uint32_t)best;
            if (w >= d.N) w -= d.N;
            return (long long)w;
        }
    }
    return -1;
}

__device__ void sym_word(const SymSlot &d, uint32_t x, uint64_t &pk)
{
    pk = 0;
    for (int j = 0; j < d.NR; j++) pk = cov_setnib(pk, j, (int)((x / d.pw[j]) % (uint32_t)d.q));
}

// emit an op: every CTA runs it after the next cluster barrier
__device__ __forceinline__ void sym_emit(SymSmem &S, int op, int i, int p, int v, int sign)
{
    S.op = op; S.oi = i; S.opos = p; S.oval = v; S.osign = sign;
    S.acc = 0ull;
    S.t_mark = sym_clock();
}

__device__ bool sym_should_stop(const SymSlot &d, SymSmem &S)
{
    const int st = cov_ldcg(&d.st->status);
    if (st && !S.status) S.status = st;
    if (S.status) return true;
    if ((unsigned long long)sym_clock() > S.deadline) { S.status = COV_ETIMEOUT; return true; }
    return false;
}

// Plan the next iteration up to its estimate op (symsearch.c:376-435).
// Returns false when the run stops.
__device__ bool sym_plan_move(const SymSlot &d, SymSmem &S)
{
    const int tid = threadIdx.x;
    const int q = d.q, NR = d.NR, R = d.R, norb = d.norb;
    if (tid == 0) {
        int stop = sym_should_stop(d, S) || S.unc <= 0 || S.moves_left <= 0 ||
                   (S.it_limit >= 0 && S.it >= S.it_limit);
        S.ibc[1] = stop;
        if (!stop) {
            S.it++;
            memset(&S.rec, 0, sizeof S.rec);
            S.rec.it = S.it;
        }
    }
    sym_bar();
    if (S.ibc[1]) return false;
    long long tp = sym_clock();
    const long long uw = sym_pick(d, S);
    if (tid == 0) { const long long t1 = sym_clock(); S.prof[0] += t1 - tp; tp = t1; }
    if (uw < 0) {
        if (tid == 0) { S.it--; S.status = COV_EDRIFT; }
        sym_bar();
        return false;
    }
    uint64_t u;
    sym_word(d, (uint32_t)uw, u);
    // effective distance of every (orbit, delta) centre and the target
    const int npair = norb * q;
    int dm = 0x7fffffff;
    for (int t = tid; t < npair; t += SNT) {
        const int i = t / q, dl = t - i * q;
        if (R - (dl != 0) < 0) continue;
        const uint64_t e = cov_ldcg(&d.rep[i]);
        int dd = 0;
        for (int j = 0; j < NR; j++) dd += sym_cdig(d, e, dl, j) != cov_nib(u, j);
        dm = min(dm, dd + (dl != 0));
    }
    dm = sym_block_min(S, dm);
    const int dtar = dm <= R + 1 ? R + 1 : dm;
    // candidates in (orbit, delta, position) order (symsearch.c:406-418)
    int nc = 0;
    for (int t0 = 0; t0 < npair; t0 += SNT) {
        const int t = t0 + tid;
        int cntc = 0, i = 0, dl = 0;
        uint64_t e = 0;
        if (t < npair) {
            i = t / q; dl = t - i * q;
            if (R - (dl != 0) >= 0) {
                e = cov_ldcg(&d.rep[i]);
                int dd = 0;
                for (int j = 0; j < NR; j++) dd += sym_cdig(d, e, dl, j) != cov_nib(u, j);
                if (dd + (dl != 0) == dtar) cntc = dd;
            }
        }
        int tot;
        const int pos = sym_block_scan(S, cntc, &tot);
        if (cntc) {
            int k = nc + pos;
            for (int j = 0; j < NR; j++) {
                const int cj = sym_cdig(d, e, dl, j), uj = cov_nib(u, j);
                if (cj == uj) continue;
                int v = uj - dl;
                if (v < 0) v += q;
                const uint32_t c = ((uint32_t)i << 8) | ((uint32_t)j << 4) | (uint32_t)v;
                if (k < SYM_TS) S.cand[k] = c;
                else d.cands[k] = c;
                k++;
            }
        }
        nc += tot;
    }
    sym_bar();
    if (tid == 0) { const long long t1 = sym_clock(); S.prof[1] += t1 - tp; tp = t1; }
    // an oversized set is sampled in global memory: its head joins it there
    if (nc > SYM_TS)
        for (int k = tid; k < SYM_TS; k += SNT) d.cands[k] = S.cand[k];
    sym_bar();
    if (tid == 0) {
        if (nc == 0) {                                   // symsearch.c:419-424
            const int i = (int)(sym_mod(S, sym_draw(S), (uint64_t)norb));
            const int p = (int)(sym_mod(S, sym_draw(S), (uint64_t)NR));
            const int v = (int)(sym_mod(S, sym_draw(S), (uint64_t)q));
            const uint32_t c = ((uint32_t)i << 8) | ((uint32_t)p << 4) | (uint32_t)v;
            S.cand[0] = c;
            d.cands[0] = c;
            nc = 1;
        }
        const int take = nc < d.cand ? nc : d.cand;
        // Fisher-Yates sample (symsearch.c:425-430)
        const bool sm = nc <= SYM_TS;
        uint32_t *arr = sm ? S.cand : d.cands;
        for (int s = 0; s < take; s++) {
            const int j = s + (int)sym_mod(S, sym_draw(S), (uint64_t)(nc - s));
            const uint32_t a = arr[s];
            arr[s] = arr[j];
            arr[j] = a;
        }
        S.take = take;
        S.cand_sm = take <= SYM_TS && sm;
        S.rec.u = uw;
        S.rec.ncand = nc;
        S.rec.ncw = take;
    }
    sym_bar();
    // estimates start from zero
    for (int s = tid; s < S.take; s += SNT) cov_stcg(&d.cd[s], 0);
    if (!S.cand_sm && S.take <= SYM_TS) {
        // nc exceeded the shared list but the sample fits: bring it in
        for (int s = tid; s < S.take; s += SNT) S.cand[s] = cov_ldcg(&d.cands[s]);
    }
    sym_bar();
    if (tid == 0) {
        S.prof[2] += sym_clock() - tp;
        sym_emit(S, SOP_EVAL, 0, 0, 0, 0);
    }
    sym_bar();
    return true;
}

// Reservoir selection over the estimates (symsearch.c:436-445)
__device__ void sym_select(const SymSlot &d, SymSmem &S)
{
    const int tid = threadIdx.x, take = S.take;
    const bool sm = take <= SYM_TS;
    if (sm) {
        for (int s = tid; s < take; s += SNT) {
            const uint32_t c = S.cand[s];
            S.cdv[s] = cov_ldcg(&d.cd[s]);
            S.skip[s] = (uint8_t)((int)(c & 15u) == cov_nib(cov_ldcg(&d.rep[c >> 8]), (int)((c >> 4) & 15u)));
        }
    }
    sym_bar();
    if (tid == 0) {
        int bs = -1, nties = 0;
        long long bestd = 1LL << 60;
        for (int s = 0; s < take; s++) {
            int cd, sk;
            if (sm) { cd = S.cdv[s]; sk = S.skip[s]; }
            else {
                const uint32_t c = cov_ldcg(&d.cands[s]);
                cd = cov_ldcg(&d.cd[s]);
                sk = (int)(c & 15u) == cov_nib(cov_ldcg(&d.rep[c >> 8]), (int)((c >> 4) & 15u));
            }
            if (sk) continue;
            if (cd < bestd) { bestd = cd; bs = s; nties = 1; }
            else if (cd == bestd) {
                nties++;
                if (sym_mod(S, sym_draw(S), (uint64_t)nties) == 0) bs = s;
            }
        }
        uint32_t c;
        int i, p, v;
        if (bs >= 0) {
            c = sm ? S.cand[bs] : cov_ldcg(&d.cands[bs]);
            i = (int)(c >> 8); p = (int)((c >> 4) & 15u); v = (int)(c & 15u);
        } else {
            bs = (int)(sym_mod(S, sym_draw(S), (uint64_t)take));
            c = sm ? S.cand[bs] : cov_ldcg(&d.cands[bs]);
            i = (int)(c >> 8); p = (int)((c >> 4) & 15u); v = (int)(c & 15u);
            if (v == cov_nib(cov_ldcg(&d.rep[i]), p)) v = (v + 1) % d.q;
        }
        S.est = sm ? S.cdv[bs] : cov_ldcg(&d.cd[bs]);
        S.rec.i = i; S.rec.p = p; S.rec.v = v; S.rec.delta = S.est;
        sym_emit(S, SOP_COMMIT, i, p, v, 0);
    }
    sym_bar();
}

__device__ void sym_copy_best(const SymSlot &d)
{
    for (int i = threadIdx.x; i < d.norb; i += SNT) cov_stcg(&d.best[i], cov_ldcg(&d.rep[i]));
}

// close the iteration: trace record, budget
__device__ void sym_finish_iter(const SymSlot &d, SymSmem &S)
{
    if (threadIdx.x == 0) {
        S.rec.unc_end = S.unc;
        S.rec.best = S.best_unc;
        if (d.trace && S.trace_n < d.trace_cap) d.trace[S.trace_n] = S.rec;
        if (d.trace) S.trace_n++;
        S.moves_left--;
        S.prof[8]++;
        if (S.best_unc == 0) S.finished = 1;
    }
}

// The leader's step: consume the result of the last op, decide the next.
// Leaves S.op set (SOP_STOP ends the launch).
__device__ void sym_leader(const SymSlot &d, SymSmem &S, int mode)
{
    const int tid = threadIdx.x;
    if (tid == 0 && S.op > 0) {
        // the op just run, timed from its emission
        const long long dt = sym_clock() - S.t_mark;
        S.prof[S.op == SOP_EVAL ? 3 : S.op == SOP_COMMIT ? 5 : 6] += dt;
    }
    for (;;) {
        const int ph = S.phase;
        if (ph == SPH_INIT) {
            // greedy orbit placement (symsearch.c:340-356)
            if (tid == 0 && S.init_i > 0 && S.op == SOP_ORBIT) S.unc += (long long)S.acc;
            sym_bar();
            if (S.init_i >= d.norb) {
                sym_copy_best(d);
                if (tid == 0) { S.best_unc = S.unc; S.phase = SPH_MOVE; S.op = -1; }
                sym_bar();
                if (mode == SMODE_INIT) {
                    if (tid == 0) { S.phase = SPH_MOVE; sym_emit(S, SOP_STOP, 0, 0, 0, 0); }
                    sym_bar();
                    return;
                }
                continue;
            }
            if (tid == 0) S.ibc[1] = sym_should_stop(d, S);
            sym_bar();
            if (S.ibc[1]) {
                if (tid == 0) sym_emit(S, SOP_STOP, 0, 0, 0, 0);
                sym_bar();
                return;
            }
            long long w = sym_pick(d, S);
            if (tid == 0) {
                if (w < 0) w = (long long)sym_modN(d, sym_draw(S));
                uint64_t pk;
                sym_word(d, (uint32_t)w, pk);
                cov_stcg(&d.rep[S.init_i], pk);
                sym_emit(S, SOP_ORBIT, S.init_i, 0, 0, +1);
                S.init_i++;
            }
            sym_bar();
            return;
        }
        if (ph == SPH_MOVE) {
            if (!sym_plan_move(d, S)) {
                if (tid == 0) sym_emit(S, SOP_STOP, 0, 0, 0, 0);
                sym_bar();
                return;
            }
            if (S.split) {
                // the estimates run as a grid-wide launch: hand the sample
                // over and end this launch
                if (S.take <= SYM_TS)
                    for (int x = tid; x < S.take; x += SNT) cov_stcg(&d.cands[x], S.cand[x]);
                if (tid == 0) {
                    S.phase = SPH_SELECT;
                    S.eval_pending = 1;
                    sym_emit(S, SOP_STOP, 0, 0, 0, 0);
                }
                sym_bar();
                return;
            }
            if (tid == 0) S.phase = SPH_SELECT;
            sym_bar();
            return;
        }
        if (ph == SPH_EVAL) {
            // a move left planned for a grid-wide estimate, continued here
            for (int x = tid; x < S.take; x += SNT) cov_stcg(&d.cd[x], 0);
            sym_bar();
            if (tid == 0) { sym_emit(S, SOP_EVAL, 0, 0, 0, 0); S.phase = SPH_SELECT; }
            sym_bar();
            return;
        }
        if (ph == SPH_SELECT) {
            const long long ts = sym_clock();
            sym_select(d, S);
            if (tid == 0) S.prof[4] += sym_clock() - ts;
            if (tid == 0) S.phase = SPH_AFTER_COMMIT;
            sym_bar();
            return;
        }
        if (ph == SPH_AFTER_COMMIT) {
            if (tid == 0) {
                const uint64_t e = cov_ldcg(&d.rep[S.oi]);
                cov_stcg(&d.rep[S.oi], cov_setnib(e, S.opos, S.oval));
                S.unc += (long long)S.acc;
                S.rec.unc = S.unc;
                S.ibc[2] = 0;
                if (S.unc < S.best_unc) {                // symsearch.c:449-458
                    S.best_unc = S.unc;
                    S.since_improve = 0;
                    S.ibc[2] = 1;
                } else if (++S.since_improve > d.stall) {
                    S.ibc[2] = 2;
                    S.kick_t = 0;
                }
            }
            sym_bar();
            if (S.ibc[2] == 1) sym_copy_best(d);
            if (S.ibc[2] == 2 && d.kick > 0) {
                if (tid == 0) S.phase = SPH_KICK_DEL;
                sym_bar();
                continue;
            }
            if (S.ibc[2] == 2) {
                if (tid == 0) { S.nkicks++; S.since_improve = 0; S.rec.kicked = 1; }
                sym_bar();
            }
            sym_finish_iter(d, S);
            if (tid == 0) S.phase = SPH_MOVE;
            sym_bar();
            continue;
        }
        if (ph == SPH_KICK_DEL) {
            // kick: take an orbit off ... (symsearch.c:459-475)
            if (tid == 0) {
                const int i = (int)(sym_mod(S, sym_draw(S), (uint64_t)d.norb));
                sym_emit(S, SOP_ORBIT, i, 0, 0, -1);
                S.phase = SPH_KICK_ADD;
            }
            sym_bar();
            return;
        }
        if (ph == SPH_KICK_ADD) {
            // ... and put it back near an uncovered word
            if (tid == 0) S.unc += (long long)S.acc;
            sym_bar();
            const long long w = sym_pick(d, S);
            if (tid == 0) {
                const int i = S.oi;
                uint64_t pk = 0;
                if (w >= 0) {
                    sym_word(d, (uint32_t)w, pk);
                    for (int t2 = 0; t2 < d.R; t2++) {
                        // the value is drawn before the position, as gcc
                        // sequences symsearch.c:467
                        const int val = (int)(sym_mod(S, sym_draw(S), (uint64_t)d.q));
                        const int pos = (int)(sym_mod(S, sym_draw(S), (uint64_t)d.NR));
                        pk = cov_setnib(pk, pos, val);
                    }
                } else {
                    for (int j = 0; j < d.NR; j++) pk = cov_setnib(pk, j, (int)(sym_mod(S, sym_draw(S), (uint64_t)d.q)));
                }
                cov_stcg(&d.rep[i], pk);
                sym_emit(S, SOP_ORBIT, i, 0, 0, +1);
                S.phase = SPH_KICK_NEXT;
            }
            sym_bar();
            return;
        }
        if (ph == SPH_KICK_NEXT) {
            if (tid == 0) {
                S.unc += (long long)S.acc;
                S.kick_t++;
                S.phase = S.kick_t < d.kick ? SPH_KICK_DEL : SPH_DONE;
            }
            sym_bar();
            continue;
        }
        if (ph == SPH_DONE) {
            if (tid == 0) { S.nkicks++; S.since_improve = 0; S.rec.kicked = 1; }
            sym_bar();
            sym_finish_iter(d, S);
            if (tid == 0) S.phase = SPH_MOVE;
            sym_bar();
            continue;
        }
        if (tid == 0) { S.status = COV_ESTATE; sym_emit(S, SOP_STOP, 0, 0, 0, 0); }
        sym_bar();
        return;
    }
}

__global__ void __launch_bounds__(SNT, 1)
sym_kernel(const SymSlot *slots, const int *list, int mode, unsigned long long budget_ns, long long op_guard,
           int split)
{
    extern __shared__ __align__(16) unsigned char sym_raw[];
    SymSmem &S = *reinterpret_cast<SymSmem *>(sym_raw);
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int sidx = list[blockIdx.x / csize];
    if (threadIdx.x == 0) S.slot = slots[sidx];
    sym_bar();
    const SymSlot &d = S.slot;
    SymSmem *LS = cl.map_shared_rank(&S, 0);
    if (rank == 0)
        for (int m = threadIdx.x + 1; m <= SYM_INV; m += SNT) S.inv[m] = ~0ull / (uint64_t)m;
    if (rank == 0 && threadIdx.x == 0) {
        const SymState &st = *d.st;
        for (int k = 0; k < 4; k++) S.rng.s[k] = st.rng[k];
        S.it = st.it; S.unc = st.unc; S.best_unc = st.best_unc; S.since_improve = st.since_improve;
        S.nkicks = st.nkicks; S.trace_n = st.trace_n; S.moves_left = st.moves_left; S.it_limit = st.it_limit;
        S.init_i = st.init_i; S.status = st.status; S.finished = st.finished;
        for (int k = 0; k < 9; k++) S.prof[k] = st.prof[k];
        S.phase = S.init_i < d.norb ? SPH_INIT : SPH_MOVE;
        S.op = -1;
        S.guard = 0;
        S.deadline = (unsigned long long)sym_clock() + budget_ns * SYM_CYCLES_PER_NS;
        if (S.status) S.phase = SPH_MOVE;
        S.split = split;
        S.eval_pending = st.eval_pending;
        if (st.eval_pending) {
            // the estimates of this move were left to a grid-wide launch
            // (already run when this launch is split too)
            S.take = st.take;
            S.rec = st.rec;
            S.phase = split ? SPH_SELECT : SPH_EVAL;
            S.eval_pending = 0;
        }
    }
    sym_bar();
    if (rank == 0 && S.phase == SPH_SELECT && S.take <= SYM_TS)
        for (int x = threadIdx.x; x < S.take; x += SNT) S.cand[x] = cov_ldcg(&d.cands[x]);
    if (rank == 0 && S.phase == SPH_EVAL && S.take <= SYM_TS)
        for (int x = threadIdx.x; x < S.take; x += SNT) S.cand[x] = cov_ldcg(&d.cands[x]);
    sym_bar();
    for (;;) {
        if (rank == 0) {
            if (S.status && S.phase != SPH_MOVE) {
                if (threadIdx.x == 0) sym_emit(S, SOP_STOP, 0, 0, 0, 0);
                sym_bar();
            } else {
                sym_leader(d, S, mode);
            }
            if (threadIdx.x == 0 && ++S.guard > op_guard && S.op != SOP_STOP) {
                S.status = COV_ESTATE;
                S.op = SOP_STOP;
            }
            sym_bar();
        }
        cl.sync();
        const int op = LS->op, oi = LS->oi, opos = LS->opos, oval = LS->oval, osign = LS->osign;
        const int take = LS->take;
        if (op == SOP_STOP) break;
        if (op == SOP_ORBIT) sym_op_orbit(d, S, LS, cl, rank, csize, oi, osign);
        else if (op == SOP_EVAL) sym_op_eval(d, S, LS, rank, csize, take);
        else if (op == SOP_COMMIT) sym_op_commit(d, S, LS, cl, rank, csize, oi, opos, oval);
        cl.sync();
    }
    if (rank == 0 && threadIdx.x == 0) {
        SymState &st = *d.st;
        for (int k = 0; k < 4; k++) st.rng[k] = S.rng.s[k];
        st.it = S.it; st.unc = S.unc; st.best_unc = S.best_unc; st.since_improve = S.since_improve;
        st.nkicks = S.nkicks; st.trace_n = S.trace_n; st.moves_left = S.moves_left;
        st.init_i = S.init_i;
        for (int k = 0; k < 9; k++) st.prof[k] = S.prof[k];
        st.eval_pending = S.eval_pending;
        st.take = S.take;
        st.rec = S.rec;
        if (S.status) atomicCAS(&st.status, 0, S.status);
        st.finished = S.finished || S.unc <= 0;
    }
}

// The estimates of one instance's planned move over the whole grid
// (symsearch.c:432-433 for every sampled candidate); the cluster kernel left
// the sample in cands[0..take) and zeroed cd[0..take).
__global__ void __launch_bounds__(SNT, 1) sym_eval_kernel(const SymSlot *slots, int slot)
{
    extern __shared__ __align__(16) unsigned char sym_raw[];
    SymSmem &S = *reinterpret_cast<SymSmem *>(sym_raw);
    if (threadIdx.x == 0) S.slot = slots[slot];
    sym_bar();
    const SymSlot &d = S.slot;
    if (!cov_ldcg(&d.st->eval_pending) || cov_ldcg(&d.st->status)) return;
    const int take = cov_ldcg(&d.st->take);
    if (take <= SYM_TS) {
        for (int x = threadIdx.x; x < take; x += SNT) S.cand[x] = cov_ldcg(&d.cands[x]);
        sym_bar();
    }
    sym_eval_items<true>(d, S, (int)blockIdx.x, (int)gridDim.x, take);
}

__global__ void k_sym_budget(SymState *states, const int *list, int count, long long moves)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) {
        SymState &s = states[list[k]];
        long long m = moves;
        if (s.it_limit >= 0) m = min(m, max(0ll, s.it_limit - s.it));
        s.moves_left = m;
    }
}

__global__ void k_sym_unpack(const uint32_t *cnt2, uint32_t N, uint16_t *out)
{
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
        out[x] = reinterpret_cast<const unsigned short *>(cnt2)[x];
}

// =========================================================== host side =====
#define SCK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "covgpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
    return -(100 + (int)e_); } } while (0)

namespace {

long long s_ipow(long long b, int e) { long long r = 1; while (e-- > 0) r *= b; return r; }
long long s_binom(int a, int b)
{
    if (b < 0 || b > a) return 0;
    if (b > a - b) b = a - b;
    long long r = 1;
    for (int i = 0; i < b; i++) r = r * (a - i) / (i + 1);
    return r;
}

// lexicographic r-subsets of pool[0..np)
void s_subsets(const int *pool, int np, int r, int rs, std::vector<uint8_t> &out)
{
    const long long nc = s_binom(np, r);
    int c[16];
    for (int i = 0; i < r; i++) c[i] = i;
    for (long long k = 0; k < nc; k++) {
        for (int i = 0; i < rs; i++) out.push_back(i < r ? (uint8_t)pool[c[i]] : 0);
        int i = r - 1;
        while (i >= 0 && c[i] == np - r + i) i--;
        if (i < 0) break;
        c[i]++;
        for (int j = i + 1; j < r; j++) c[j] = c[j - 1] + 1;
    }
}

struct SymHost {
    bool used = false;
    SymSlot d{};
    void *arena = nullptr;
    int cluster = 1;
};

CovDeviceFlags g_sym_attr;   // kernel attributes set, per device

int sym_attrs()
{
    int dev = 0;
    if (g_sym_attr.done(dev)) return 0;
    SCK(cudaFuncSetAttribute(sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SymSmem)));
    SCK(cudaFuncSetAttribute(sym_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    SCK(cudaFuncSetAttribute(sym_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SymSmem)));
    g_sym_attr.set(dev);
    return 0;
}

}  // namespace

struct cov_sym {
    int max_slots = 0, cluster = 1;
    int grid_eval = 0;           // one live instance: estimates over the whole GPU
    int sms = 0;
    double budget_s = 30.0;
    std::vector<SymHost> slots;
    SymSlot *d_slots = nullptr;
    SymState *d_states = nullptr;
    int *d_list = nullptr;
    cudaStream_t stream = nullptr;
};

static int sym_push(cov_sym *p, int s)
{
    SCK(cudaMemcpyAsync(p->d_slots + s, &p->slots[s].d, sizeof(SymSlot), cudaMemcpyHostToDevice, p->stream));
    return 0;
}

// one launch per cluster size over the listed live slots
static int sym_launch(cov_sym *p, const std::vector<int> &slots, int mode, long long moves)
{
    std::vector<int> sizes;
    for (int s : slots) sizes.push_back(p->slots[s].cluster);
    std::sort(sizes.begin(), sizes.end());
    sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
    int kmax = 0, omax = 0;
    for (int s : slots) {
        kmax = std::max(kmax, p->slots[s].d.kick);
        omax = std::max(omax, p->slots[s].d.norb);
    }
    const long long guard = moves * (4 + 3LL * kmax) + 2LL * omax + 4096;
    const unsigned long long budget_ns = (unsigned long long)(p->budget_s * 1e9);
    for (int cs : sizes) {
        std::vector<int> list;
        for (int s : slots) if (p->slots[s].cluster == cs) list.push_back(s);
        SCK(cudaMemcpyAsync(p->d_list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, p->stream));
        if (mode == SMODE_RUN) {
            k_sym_budget<<<(unsigned)((list.size() + 127) / 128), 128, 0, p->stream>>>(p->d_states, p->d_list,
                                                                                   (int)list.size(), moves);
            SCK(cudaGetLastError());
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(list.size() * cs));
        cfg.blockDim = dim3(SNT);
        cfg.dynamicSmemBytes = sizeof(SymSmem);
        cfg.stream = p->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (mode == SMODE_RUN && p->grid_eval && slots.size() == 1) {
            // one instance: each move is a cluster launch up to the
            // estimates and a grid-wide launch for them; moves + 1 cluster
            // launches close the last move (a finished instance's extra
            // launches return at once)
            for (long long m = 0; m <= moves; m++) {
                SCK(cudaLaunchKernelEx(&cfg, sym_kernel, (const SymSlot *)p->d_slots, (const int *)p->d_list,
                                       mode, budget_ns, guard, 1));
                if (m < moves) {
                    sym_eval_kernel<<<(unsigned)p->sms, SNT, sizeof(SymSmem), p->stream>>>(
                        (const SymSlot *)p->d_slots, slots[0]);
                }
                SCK(cudaGetLastError());
            }
        } else {
            SCK(cudaLaunchKernelEx(&cfg, sym_kernel, (const SymSlot *)p->d_slots, (const int *)p->d_list, mode,
                                   budget_ns, guard, 0));
            SCK(cudaGetLastError());
        }
        SCK(cudaStreamSynchronize(p->stream));
    }
    return 0;
}

extern "C" {

int cov_sym_create(int32_t max_slots, int32_t cluster, cov_sym **out)
{
    if (!out || max_slots < 1 || max_slots > 65536 || cluster < 1 || cluster > 16) return COV_EINVAL;
    *out = nullptr;
    int dev = 0, major = 0;
    SCK(cudaGetDevice(&dev));
    SCK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major < 10) return COV_ENODEV;
    int rc = sym_attrs();
    if (rc) return rc;
    cov_sym *p = new cov_sym();
    p->max_slots = max_slots;
    p->cluster = cluster;
    p->slots.resize(max_slots);
    SCK(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev));
    cudaError_t e = cudaMalloc(&p->d_slots, sizeof(SymSlot) * max_slots);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_states, sizeof(SymState) * max_slots);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_list, sizeof(int) * max_slots);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaFree(p->d_slots); cudaFree(p->d_states); cudaFree(p->d_list);
        delete p;
        return -(100 + (int)e);
    }
    *out = p;
    return COV_OK;
}

int cov_sym_destroy(cov_sym *p)
{
    if (!p) return COV_EINVAL;
    cudaStreamSynchronize(p->stream);
    for (auto &h : p->slots) if (h.used) cudaFree(h.arena);
    cudaFree(p->d_slots); cudaFree(p->d_states); cudaFree(p->d_list);
    cudaStreamDestroy(p->stream);
    delete p;
    return COV_OK;
}

int cov_sym_set_budget(cov_sym *p, double seconds)
{
    if (!p || !(seconds > 0)) return COV_EINVAL;
    p->budget_s = seconds;
    return COV_OK;
}

// Pool setting: "grid_eval" 1 runs a pool with one live instance with its
// estimates spread over the whole GPU (a launch per move for them), 0 (the
// default) keeps every move inside the instance's cluster.  Neither
// changes a trajectory.
int cov_sym_set_param(cov_sym *p, const char *name, int64_t value)
{
    if (!p || !name) return COV_EINVAL;
    if (!strcmp(name, "grid_eval")) {
        if (value < 0 || value > 1) return COV_EINVAL;
        p->grid_eval = (int)value;
        return COV_OK;
    }
    return COV_EINVAL;
}

int cov_sym_orbits(const cov_sym_params *prm)
{
    if (!prm) return COV_EINVAL;
    const int q = prm->q, n = prm->n, R = prm->R, M = prm->M;
    if (q < 2 || n < 2 || R < 0 || R > SYM_MAXR || M < q) return COV_EINVAL;      // symsearch exit 2
    const int norb = prm->orbits > 0 ? prm->orbits : M / q;
    if (norb < 1 || norb > M / q) return COV_ERANGE;                              // exit 3
    if (q > 16 || n > 16) return COV_EINVAL;
    if (s_ipow(q, n - 1) > 4000000000LL) return COV_ERANGE;
    if ((long long)norb * q > 65000) return COV_ERANGE;
    return norb;
}

size_t cov_sym_slot_bytes(const cov_sym_params *prm)
{
    const int norb = cov_sym_orbits(prm);
    if (norb <= 0) return 0;
    const int q = prm->q, NR = prm->n - 1;
    const long long N = s_ipow(q, NR);
    size_t b = 0;
    auto add = [&](size_t x) { b += (x + 255) / 256 * 256; };
    add((size_t)((N + 1) / 2) * 4);
    add((size_t)((N + 63) / 64 + 2) * 16);
    add((size_t)norb * 8 * 2);
    add(((size_t)norb * q * NR + 8) * 4 * 2);
    add(sizeof(SymState));
    if (prm->trace) add((size_t)prm->trace_cap * sizeof(cov_move_rec));
    add(65536);
    return b;
}

int cov_sym_remove(cov_sym *p, int32_t slot);

int cov_sym_add(cov_sym *p, const cov_sym_params *prm, int32_t *slot)
{
    if (!p || !prm || !slot) return COV_EINVAL;
    const int norb = cov_sym_orbits(prm);
    if (norb <= 0) return norb;
    if (prm->kick < 0 || prm->stall < 0 || prm->cand < 1 || prm->trace_cap < 0) return COV_EINVAL;
    int s = -1;
    for (int k = 0; k < p->max_slots; k++) if (!p->slots[k].used) { s = k; break; }
    if (s < 0) return COV_ERANGE;
    const int q = prm->q, n = prm->n, R = prm->R, NR = n - 1;
    SymHost h;
    h.cluster = p->cluster;
    SymSlot &d = h.d;
    d.q = q; d.n = n; d.R = R; d.NR = NR; d.norb = norb;
    d.N = (uint32_t)s_ipow(q, NR);
    for (int j = 0; j < NR; j++) d.pw[j] = (uint32_t)s_ipow(q, NR - 1 - j);
    for (int k = 0; k <= COV_MAXN; k++) d.ppow[k] = (uint32_t)std::min<long long>(s_ipow(q - 1, k), 0xffffffffLL);
    d.kick = prm->kick; d.cand = prm->cand; d.stall = prm->stall;
    d.rs = R ? R : 1;
    // walk subsets: radius R and R-1, positions other than p
    std::vector<uint8_t> w0, w1, bs;
    for (int t = 0; t < 2; t++) {
        const int rad = R - t;
        std::vector<uint8_t> &out = t ? w1 : w0;
        d.wnc[t] = rad >= 0 ? (int)s_binom(NR - 1, rad) : 0;
        for (int pp = 0; pp < NR && rad >= 0; pp++) {
            int pool[32], np = 0;
            for (int j = 0; j < NR; j++) if (j != pp) pool[np++] = j;
            s_subsets(pool, np, rad, d.rs, out);
        }
        if (out.empty()) out.push_back(0);
        if (rad < 0) d.witems[t] = 0;
        else if (rad == 0) d.witems[t] = 1;
        else d.witems[t] = (uint32_t)((long long)d.wnc[t] * s_ipow(q - 1, rad - 1));
    }
    d.ipc = d.witems[0] + (R >= 1 ? (uint32_t)(q - 1) * d.witems[1] : 0u);
    // ball subsets r = 1..R of all NR positions
    {
        int pool[32];
        for (int j = 0; j < NR; j++) pool[j] = j;
        int off = 0;
        d.bcum[0] = 0;
        d.bcum[1] = 0;
        for (int r = 1; r <= SYM_MAXR + 1; r++) {
            if (r <= R) {
                d.boff[r] = off;
                s_subsets(pool, NR, r, d.rs, bs);
                off += (int)s_binom(NR, r);
            }
            if (r + 1 <= SYM_MAXR + 1)
                d.bcum[r + 1] = d.bcum[r] + (r <= R ? (uint32_t)(s_binom(NR, r) * s_ipow(q - 1, r - 1)) : 0u);
        }
        if (bs.empty()) bs.push_back(0);
        d.bitems[0] = 1 + d.bcum[std::min(R, SYM_MAXR) + 1];
        d.bitems[1] = R >= 1 ? 1 + d.bcum[R] : 0;
        d.opi = d.bitems[0] + (R >= 1 ? (uint32_t)(q - 1) * d.bitems[1] : 0u);
    }
    // reciprocals for multiply-high division (exact: x < 2^24 for q-1,
    // x < 2^32 for the 64-bit ones)
    auto inv64 = [](uint64_t m) -> uint64_t { return m <= 1 ? 0 : ~0ull / m + 1; };
    d.inv_qm1 = q > 2 ? (uint32_t)(0xffffffffull / (uint64_t)(q - 1) + 1) : 0u;
    for (int k = 0; k <= SYM_MAXR; k++) d.inv_pp[k] = inv64(d.ppow[k]);
    d.inv_wit1 = inv64(d.witems[1]);
    d.inv_bit1 = inv64(d.bitems[1]);
    d.inv_ipc = inv64(d.ipc);
    d.inv_N = ~0ull / (uint64_t)d.N;
    const size_t ncap = (size_t)norb * q * NR + 8;
    const size_t need = cov_sym_slot_bytes(prm) + w0.size() + w1.size() + bs.size() + 1024;
    void *arena = nullptr;
    if (cudaMalloc(&arena, need) != cudaSuccess) { cudaGetLastError(); return COV_ENOMEM; }
    size_t off = 0;
    auto take_ = [&](size_t x) { void *q2 = (char *)arena + off; off += (x + 255) / 256 * 256; return q2; };
    d.cnt2 = (uint32_t *)take_((size_t)((d.N + 1) / 2) * 4);
    d.st2 = (uint32_t *)take_((size_t)((d.N + 63) / 64 + 2) * 16);
    d.rep = (uint64_t *)take_((size_t)norb * 8);
    d.best = (uint64_t *)take_((size_t)norb * 8);
    d.cands = (uint32_t *)take_(ncap * 4);
    d.cd = (int32_t *)take_(ncap * 4);
    uint8_t *dw0 = (uint8_t *)take_(w0.size());
    uint8_t *dw1 = (uint8_t *)take_(w1.size());
    uint8_t *dbs = (uint8_t *)take_(bs.size());
    d.wsub[0] = dw0; d.wsub[1] = dw1; d.bsub = dbs;
    d.trace = prm->trace ? (cov_move_rec *)take_((size_t)prm->trace_cap * sizeof(cov_move_rec)) : nullptr;
    d.trace_cap = prm->trace ? prm->trace_cap : 0;
    d.st = p->d_states + s;
    SymState st{};
    CovRng r;
    cov_rng_seed(r, prm->seed * 0x9E3779B97F4A7C15ULL + 12345ULL);     // symsearch.c:338
    for (int k = 0; k < 4; k++) st.rng[k] = r.s[k];
    st.unc = d.N;
    st.best_unc = d.N;
    st.it_limit = -1;
    cudaError_t e = cudaMemsetAsync(d.cnt2, 0, (size_t)((d.N + 1) / 2) * 4, p->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.st2, 0, (size_t)((d.N + 63) / 64 + 2) * 16, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw0, w0.data(), w0.size(), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw1, w1.data(), w1.size(), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dbs, bs.data(), bs.size(), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.st, &st, sizeof st, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) { cudaFree(arena); return -(100 + (int)e); }
    h.arena = arena;
    h.used = true;
    p->slots[s] = h;
    int rc = sym_push(p, s);
    // greedy initialisation on the device
    if (!rc) rc = sym_launch(p, std::vector<int>{s}, SMODE_INIT, 0);
    if (rc) {
        cov_sym_remove(p, s);
        return rc;
    }
    *slot = s;
    return COV_OK;
}

int cov_sym_remove(cov_sym *p, int32_t slot)
{
    if (!p || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    SCK(cudaStreamSynchronize(p->stream));
    cudaFree(p->slots[slot].arena);
    p->slots[slot] = SymHost();
    return COV_OK;
}

int cov_sym_set_slot_param(cov_sym *p, int32_t slot, const char *name, int64_t value)
{
    if (!p || !name || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    if (!strcmp(name, "cluster")) {
        if (value < 1 || value > 16) return COV_EINVAL;
        p->slots[slot].cluster = (int)value;
        return COV_OK;
    }
    if (!strcmp(name, "it_limit")) {
        if (value < -1) return COV_EINVAL;
        long long v = value;
        SCK(cudaMemcpyAsync(&p->slots[slot].d.st->it_limit, &v, sizeof v, cudaMemcpyHostToDevice, p->stream));
        SCK(cudaStreamSynchronize(p->stream));
        return COV_OK;
    }
    return COV_EINVAL;
}

int cov_sym_run(cov_sym *p, int64_t moves)
{
    if (!p || moves < 0) return COV_EINVAL;
    std::vector<int> live;
    for (int s = 0; s < p->max_slots; s++) if (p->slots[s].used) live.push_back(s);
    if (live.empty() || moves == 0) return COV_OK;
    return sym_launch(p, live, SMODE_RUN, moves);
}

int cov_sym_status(cov_sym *p, int32_t slot, cov_status *out)
{
    if (!p || !out || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    SymState st;
    SCK(cudaMemcpyAsync(&st, p->slots[slot].d.st, sizeof st, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    out->it = st.it; out->uncovered = st.unc; out->best = st.best_unc; out->kicks = st.nkicks;
    out->trace_n = st.trace_n; out->status = st.status; out->finished = st.finished;
    out->ul_valid = 0; out->ul_n = 0;
    return COV_OK;
}

int cov_sym_resume(cov_sym *p, int32_t slot)
{
    if (!p || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    int st = 0;
    SCK(cudaMemcpyAsync(&st, &p->slots[slot].d.st->status, sizeof st, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    if (st != COV_ETIMEOUT) return st ? COV_ESTATE : COV_OK;
    st = 0;
    SCK(cudaMemcpyAsync(&p->slots[slot].d.st->status, &st, sizeof st, cudaMemcpyHostToDevice, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    return COV_OK;
}

static int sym_get_reps(cov_sym *p, int32_t slot, bool best, uint8_t *out)
{
    if (!p || !out || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    const SymSlot &d = p->slots[slot].d;
    std::vector<uint64_t> pk(d.norb);
    SCK(cudaMemcpyAsync(pk.data(), best ? d.best : d.rep, pk.size() * 8, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    for (int i = 0; i < d.norb; i++)
        for (int j = 0; j < d.NR; j++) out[(size_t)i * d.NR + j] = (uint8_t)cov_nib(pk[i], j);
    return COV_OK;
}

int cov_sym_get_rep(cov_sym *p, int32_t slot, uint8_t *out) { return sym_get_reps(p, slot, false, out); }
int cov_sym_get_best(cov_sym *p, int32_t slot, uint8_t *out) { return sym_get_reps(p, slot, true, out); }

int cov_sym_get_cnt(cov_sym *p, int32_t slot, uint16_t *out)
{
    if (!p || !out || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    const SymSlot &d = p->slots[slot].d;
    uint16_t *tmp = nullptr;
    if (cudaMalloc(&tmp, (size_t)d.N * 2) != cudaSuccess) { cudaGetLastError(); return COV_ENOMEM; }
    k_sym_unpack<<<1024, 256, 0, p->stream>>>(d.cnt2, d.N, tmp);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, (size_t)d.N * 2, cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return -(100 + (int)e);
    return COV_OK;
}

int cov_sym_get_trace(cov_sym *p, int32_t slot, cov_move_rec *out, int64_t cap, int64_t *n_out)
{
    if (!p || !n_out || (!out && cap > 0) || slot < 0 || slot >= p->max_slots || !p->slots[slot].used)
        return COV_EINVAL;
    const SymSlot &d = p->slots[slot].d;
    SymState st;
    SCK(cudaMemcpyAsync(&st, d.st, sizeof st, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    const long long have = std::min<long long>(st.trace_n, d.trace_cap);
    if (!out) { *n_out = have > 0 ? have : 0; return COV_OK; }
    const long long n = std::min<long long>(have, cap);
    if (n > 0 && d.trace) {
        SCK(cudaMemcpyAsync(out, d.trace, (size_t)n * sizeof(cov_move_rec), cudaMemcpyDeviceToHost, p->stream));
        SCK(cudaStreamSynchronize(p->stream));
    }
    *n_out = n > 0 ? n : 0;
    return COV_OK;
}

int cov_sym_get_prof(cov_sym *p, int32_t slot, uint64_t *out)
{
    if (!p || !out || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    SymState st;
    SCK(cudaMemcpyAsync(&st, p->slots[slot].d.st, sizeof st, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    for (int k = 0; k < 9; k++) out[k] = st.prof[k];
    return COV_OK;
}

int cov_sym_get_rng(cov_sym *p, int32_t slot, uint64_t *out)
{
    if (!p || !out || slot < 0 || slot >= p->max_slots || !p->slots[slot].used) return COV_EINVAL;
    SymState st;
    SCK(cudaMemcpyAsync(&st, p->slots[slot].d.st, sizeof st, cudaMemcpyDeviceToHost, p->stream));
    SCK(cudaStreamSynchronize(p->stream));
    for (int k = 0; k < 4; k++) out[k] = st.rng[k];
    return COV_OK;
}

}  // extern "C"
