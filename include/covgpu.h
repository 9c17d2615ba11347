/*
 * covgpu.h -- C ABI of libcovgpu.so, the GB300 (sm_103a) covering-code
 * search and verification library.
 *
 * Conventions (kept from the reference's own C-ABI libraries,
 * cov/gemm2/dct.cu:55-57 and cov/gemm2/chainsolve.cu:370-433):
 *   - every entry point returns int: 0 = ok, negative = error;
 *     -(100 + cudaError_t) for a CUDA runtime error;
 *   - host buffers are plain pointers owned by the caller; the library owns
 *     device memory between *_create and *_destroy;
 *   - the library spawns no threads; one caller thread per handle.
 * Codewords are uint8 digits, MSB first: word index x = sum_j w_j q^(n-1-j)
 * (cov/engine/covsearch2e.c:916-921, cov/verify_cov.py:27-35).
 *
 * Domain (the reference engine's own limits, covsearch2e.c:1111-1117, and
 * this library's packing): 2 <= q <= 16, 1 <= n <= 16, 0 <= R,
 * q^n < 2^32, 1 <= M <= 65535.
 */
#ifndef COVGPU_H
#define COVGPU_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COV_OK              0
#define COV_EINVAL         -1   /* bad parameter / outside the domain       */
#define COV_ENOMEM         -2   /* device allocation failed                  */
#define COV_ESTATE         -3   /* call out of order (e.g. run before load)  */
#define COV_ETIMEOUT       -4   /* a bounded device-side wait gave up        */
#define COV_EDRIFT         -5   /* an in-kernel invariant check failed       */
#define COV_ENODEV         -6   /* no usable sm_103 device                   */
#define COV_ERANGE         -7   /* request exceeds a fixed capacity          */

/* One record per tabu move; the oracle writes the same layout, so traces of
 * the two compare byte for byte.  Fields follow the per-iteration steps of
 * cov/engine/covsearch2e.c:1304-1580. */
typedef struct {
    int64_t it;         /* 1-based iteration number (covsearch2e.c:1325)    */
    int64_t u;          /* index of the sampled uncovered word (:1335)      */
    int64_t delta;      /* evaluated delta of the committed move (:1476)    */
    int64_t unc;        /* uncovered count right after the commit (:1528)   */
    int64_t unc_end;    /* uncovered count at the end of the iteration,
                           i.e. after a kick when one happened (:1553-1579) */
    int64_t best;       /* best uncovered count after the iteration         */
    int32_t ncand;      /* candidate moves collected (:1359-1380)           */
    int32_t ncw;        /* distinct candidate codewords (:1458-1465)        */
    int32_t i, p, v;    /* committed move: codeword, position, new value    */
    int32_t kicked;     /* 1 when the iteration ended in a kick             */
} cov_move_rec;

#ifdef __cplusplus
}
#endif
#endif
