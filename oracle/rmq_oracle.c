/*
 * rmq_oracle.c -- CPU oracle for the batch RMQ path. TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the CPU-baseline leg of bench.py use
 * it; the product (librmq.so, the rtxrmq CLI, the Python package) never
 * links or calls it.
 *
 * Parity is pinned: the CPU tests compare these functions with the
 * reference's own cpu_rmq / cpu_rmq_idx / rmq_rmm_par(_idx), compiled from
 * the reference sources by oracle/Makefile into oracle/_ref/, through golden
 * vectors committed under tests/golden/.
 *
 * Functions:
 *  oracle_base_val / oracle_base_idx
 *      restate cpu_min / cpu_min_idx (src/cpu_methods.h:6-16, 42-53):
 *      start from A[l], replace on strict `<`, so the leftmost minimum.
 *  oracle_blocks
 *      restates RTX_blocks (alg 5 / 105) on the CPU: block minima with their
 *      leftmost argmin (kernel_min_blocks, src/device_tools.cuh:243-253;
 *      compute_min_blocks, src/rtx.h:3-22), then per query the three "rays"
 *      of __raygen__rmq_blocks (src/rtx_kernels.cu:85-180): fully covered
 *      blocks lB+1..rB-1 from the block minima, and scans of the left and
 *      right partial blocks; a query inside one block is one scan. Ties are
 *      resolved leftmost across the three parts, i.e. BASE semantics.
 *      O(bs + nb) per query; used for large-size sampled checks and as the
 *      ported CPU baseline.
 * All functions parallelise over queries with OpenMP (`nt` threads, <= 0
 * means the OpenMP default).
 */
#include "rmq_oracle.h"

#include <omp.h>
#include <stdint.h>
#include <stdlib.h>

static void set_threads(int nt) {
    if (nt > 0) omp_set_num_threads(nt);
}

static int64_t base_scan(const float *A, int64_t l, int64_t r) {
    float m = A[l];
    int64_t mi = l;
    for (int64_t i = l; i <= r; ++i) {
        if (A[i] < m) {
            m = A[i];
            mi = i;
        }
    }
    return mi;
}

int oracle_base_val(const float *A, int64_t n, const int32_t *Q, int64_t q, float *out, int nt) {
    if (!A || !Q || !out || n <= 0 || q < 0) return -1;
    set_threads(nt);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < q; ++i) {
        const int64_t l = Q[2 * i], r = Q[2 * i + 1];
        out[i] = A[base_scan(A, l, r)];
    }
    return 0;
}

int oracle_base_idx(const float *A, int64_t n, const int32_t *Q, int64_t q, int32_t *out, int nt) {
    if (!A || !Q || !out || n <= 0 || q < 0) return -1;
    set_threads(nt);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < q; ++i) {
        const int64_t l = Q[2 * i], r = Q[2 * i + 1];
        out[i] = (int32_t)base_scan(A, l, r);
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* RTX_blocks restated                                                      */

struct oracle_blocks {
    const float *A;
    int64_t n, bs, nb;
    int64_t *bmin_idx; /* leftmost argmin of each block */
};

oracle_blocks_t *oracle_blocks_build(const float *A, int64_t n, int64_t bs, int nt) {
    if (!A || n <= 0) return NULL;
    if (bs <= 0) bs = 1 << 15;
    if (bs > n) bs = n;
    oracle_blocks_t *o = (oracle_blocks_t *)malloc(sizeof(*o));
    if (!o) return NULL;
    o->A = A;
    o->n = n;
    o->bs = bs;
    o->nb = (n + bs - 1) / bs;
    o->bmin_idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)o->nb);
    if (!o->bmin_idx) {
        free(o);
        return NULL;
    }
    set_threads(nt);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < o->nb; ++b) {
        const int64_t lo = b * bs;
        const int64_t hi = (lo + bs < n ? lo + bs : n) - 1;
        o->bmin_idx[b] = base_scan(A, lo, hi);
    }
    return o;
}

void oracle_blocks_free(oracle_blocks_t *o) {
    if (!o) return;
    free(o->bmin_idx);
    free(o);
}

/* leftmost-min merge of two candidate indices (float `<`, then index) */
static int64_t pick(const float *A, int64_t a, int64_t b) {
    if (a < 0) return b;
    if (b < 0) return a;
    if (A[b] < A[a]) return b;
    if (A[a] < A[b]) return a;
    return a < b ? a : b;
}

static int64_t blocks_one(const oracle_blocks_t *o, int64_t l, int64_t r) {
    const float *A = o->A;
    const int64_t lB = l / o->bs, rB = r / o->bs;
    if (lB == rB) return base_scan(A, l, r);
    int64_t best = -1;
    if (lB < rB - 1) { /* fully covered blocks: the "middle ray" */
        int64_t m = o->bmin_idx[lB + 1];
        for (int64_t b = lB + 2; b <= rB - 1; ++b) {
            const int64_t c = o->bmin_idx[b];
            if (A[c] < A[m]) m = c;
        }
        best = m;
    }
    best = pick(A, best, base_scan(A, l, (lB + 1) * o->bs - 1)); /* left partial block */
    best = pick(A, best, base_scan(A, rB * o->bs, r));           /* right partial block */
    return best;
}

int oracle_blocks_query(const oracle_blocks_t *o, const int32_t *Q, int64_t q, float *val,
                        int32_t *idx, int nt) {
    if (!o || !Q || q < 0 || (!val && !idx)) return -1;
    set_threads(nt);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < q; ++i) {
        const int64_t k = blocks_one(o, Q[2 * i], Q[2 * i + 1]);
        if (val) val[i] = o->A[k];
        if (idx) idx[i] = (int32_t)k;
    }
    return 0;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }
