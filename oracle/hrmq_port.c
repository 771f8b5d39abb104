/*
 * hrmq_port.c -- TEST INFRASTRUCTURE (CPU baseline / oracle only).
 *
 * A restatement, in our own code, of the succinct range-minimum structure the
 * reference uses as its CPU comparator (HRMQ: Ferrada & Navarro, "Improved
 * range minimum queries", J. Discrete Algorithms 43 (2017) 72-80; the
 * reference's implementation is hrmq/RMQRMM64.cpp, GPL-2.0, not copied).
 *
 *  1. Balanced parentheses P (2n+2 bits) of the Cartesian tree of A, built
 *     with a stack: an opening parenthesis for the root, then for each A[k]
 *     a closing parenthesis for every stacked j with A[j] >= A[k] (popped),
 *     and an opening parenthesis for k; finally one closing parenthesis per
 *     element left on the stack (hrmq/RMQRMM64.cpp:196-251). The `>=` rule
 *     makes equal values resolve to the RIGHTMOST minimum, as HRMQ does;
 *     `strict` = 1 pops only on `>`, which resolves to the LEFTMOST one.
 *  2. Query (hrmq/RMQRMM64.cpp:1463-1465):
 *        RMQ(i, j) = rank1( m ) - 2,  m = rightmost position of the minimum
 *        of E'(p) = (#1 - #0 in P[0..p-1]) over p in [select1(i+2), select1(j+2)]
 *     (the opening parenthesis of the minimum's node; nothing after it in the
 *     range goes lower, ties before it are shallower ancestors' positions).
 *  3. Support structures (our own layout): P in 64-bit words (bit p = bit
 *     p%64 of word p/64, LSB first); ones before every word (rank); the
 *     position of every 256th one (select samples); per word the minimum of
 *     E' relative to the word start and its rightmost position (via 8-bit
 *     lookup tables), and a bottom-up segment tree over the words' absolute
 *     minima (the role of HRMQ's range min-max tree over its leaf blocks).
 * Queries run in parallel with OpenMP; the build is serial (the stack pass)
 * plus parallel directory construction, as in the reference.
 */
#include "rmq_oracle.h"

#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SEL_SAMPLE 256

struct hrmq_port {
    int64_t n;
    int64_t nbits;   /* 2n + 2 */
    int64_t nwords;
    uint64_t *P;
    int64_t *ones;   /* ones in words [0, w) ; nwords + 1 entries */
    int64_t *sel;    /* position of one number s*SEL_SAMPLE + 1 */
    int64_t nsel;
    int8_t *wmin;    /* min of E' inside word w, relative to E'(64 w) */
    uint8_t *wpos;   /* rightmost offset of that minimum */
    int64_t tsize;   /* leaves in the segment tree (power of two) */
    int64_t *tval;   /* segment tree: absolute min (int64), 2*tsize */
    int64_t *tword;  /* word holding the rightmost minimum */
};

/* byte tables: for byte b read LSB first, E' before bit t (t = 0..7) is
 * 2*popcount(b & ((1<<t)-1)) - t; its minimum over t, the rightmost t that
 * reaches it, and the byte's total excess. */
static int8_t T_MIN[256];
static uint8_t T_POS[256];
static int8_t T_EXC[256];
static int tables_ready = 0;

static void init_tables(void) {
    if (tables_ready) return;
    for (int b = 0; b < 256; ++b) {
        int e = 0, mn = 1 << 20, pos = 0;
        for (int t = 0; t < 8; ++t) {
            if (e <= mn) {
                mn = e;
                pos = t;
            }
            e += ((b >> t) & 1) ? 1 : -1;
        }
        T_MIN[b] = (int8_t)mn;
        T_POS[b] = (uint8_t)pos;
        T_EXC[b] = (int8_t)e;
    }
    tables_ready = 1;
}

static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

static inline int bit(const uint64_t *P, int64_t p) { return (int)((P[p >> 6] >> (p & 63)) & 1u); }

/* E'(p): excess of P[0 .. p-1] */
static inline int64_t excess_before(const hrmq_port_t *h, int64_t p) {
    const int64_t w = p >> 6;
    const int r = (int)(p & 63);
    int64_t ones = h->ones[w];
    if (r) ones += popc64(h->P[w] & ((1ull << r) - 1));
    return 2 * ones - p;
}

/* rank1(p): ones in P[0 .. p] */
static inline int64_t rank1(const hrmq_port_t *h, int64_t p) {
    const int64_t w = p >> 6;
    const int r = (int)(p & 63);
    const uint64_t mask = (r == 63) ? ~0ull : ((1ull << (r + 1)) - 1);
    return h->ones[w] + popc64(h->P[w] & mask);
}

/* select1(k): position of the k-th one (k >= 1) */
static int64_t select1(const hrmq_port_t *h, int64_t k) {
    const int64_t s = (k - 1) / SEL_SAMPLE;
    int64_t w = h->sel[s] >> 6;
    /* advance word by word (samples keep this short) */
    while (h->ones[w + 1] < k) ++w;
    int64_t need = k - h->ones[w];
    uint64_t x = h->P[w];
    for (int byte = 0; byte < 8; ++byte) {
        const int c = popc64(x & 0xffull);
        if (c >= need) {
            for (int t = 0; t < 8; ++t) {
                if ((x >> t) & 1u) {
                    if (--need == 0) return (w << 6) + byte * 8 + t;
                }
            }
        }
        need -= c;
        x >>= 8;
    }
    return -1; /* not reached */
}

/* rightmost minimum of E' over positions [a, b] inside one word; E'(a) known */
static void scan_word(const hrmq_port_t *h, int64_t a, int64_t b, int64_t ea, int64_t *best,
                      int64_t *bpos) {
    const uint64_t x = h->P[a >> 6];
    int64_t p = a, e = ea;
    /* bits until the next byte boundary */
    while (p <= b && (p & 7)) {
        if (e <= *best) {
            *best = e;
            *bpos = p;
        }
        e += ((x >> (p & 63)) & 1u) ? 1 : -1;
        ++p;
    }
    /* whole bytes */
    while (p + 7 <= b) {
        const unsigned byte = (unsigned)((x >> (p & 63)) & 0xffu);
        const int64_t m = e + T_MIN[byte];
        if (m <= *best) {
            *best = m;
            *bpos = p + T_POS[byte];
        }
        e += T_EXC[byte];
        p += 8;
    }
    /* tail bits */
    while (p <= b) {
        if (e <= *best) {
            *best = e;
            *bpos = p;
        }
        e += ((x >> (p & 63)) & 1u) ? 1 : -1;
        ++p;
    }
}

/* rightmost minimum of the per-word absolute minima over words [w1, w2] */
static void tree_query(const hrmq_port_t *h, int64_t w1, int64_t w2, int64_t *best, int64_t *bword) {
    /* collect left-side and right-side nodes so that ties resolve rightmost */
    int64_t lo = w1 + h->tsize, hi = w2 + h->tsize + 1;
    int64_t rnodes[64];
    int nr = 0;
    int64_t lbest = INT64_MAX, lword = -1;
    while (lo < hi) {
        if (lo & 1) {
            const int64_t v = h->tval[lo];
            if (v <= lbest) {
                lbest = v;
                lword = h->tword[lo];
            }
            ++lo;
        }
        if (hi & 1) rnodes[nr++] = --hi;
        lo >>= 1;
        hi >>= 1;
    }
    for (int k = nr - 1; k >= 0; --k) {
        const int64_t v = h->tval[rnodes[k]];
        if (v <= lbest) {
            lbest = v;
            lword = h->tword[rnodes[k]];
        }
    }
    if (lword >= 0 && lbest <= *best) {
        *best = lbest;
        *bword = lword;
    }
}

static int64_t rmq_excess(const hrmq_port_t *h, int64_t x, int64_t y) {
    int64_t best = INT64_MAX, bpos = -1;
    const int64_t wx = x >> 6, wy = y >> 6;
    if (wx == wy) {
        scan_word(h, x, y, excess_before(h, x), &best, &bpos);
        return bpos;
    }
    scan_word(h, x, (wx << 6) + 63, excess_before(h, x), &best, &bpos);
    if (wy - wx >= 2) {
        int64_t tb = best, tw = -1;
        tree_query(h, wx + 1, wy - 1, &tb, &tw);
        if (tw >= 0 && tb <= best) {
            best = tb;
            bpos = (tw << 6) + h->wpos[tw];
        }
    }
    scan_word(h, wy << 6, y, excess_before(h, wy << 6), &best, &bpos);
    return bpos;
}

hrmq_port_t *hrmq_port_build(const float *A, int64_t n, int strict, int nt) {
    if (!A || n <= 0) return NULL;
    init_tables();
    if (nt > 0) omp_set_num_threads(nt);
    hrmq_port_t *h = (hrmq_port_t *)calloc(1, sizeof(*h));
    if (!h) return NULL;
    h->n = n;
    h->nbits = 2 * n + 2;
    h->nwords = (h->nbits + 63) / 64 + 1; /* one spare word */
    h->P = (uint64_t *)calloc((size_t)h->nwords, sizeof(uint64_t));
    int64_t *stack = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    if (!h->P || !stack) {
        free(stack);
        hrmq_port_free(h);
        return NULL;
    }
    /* 1. the parentheses (serial stack pass); opening = 1 */
    int64_t pos = 0, top = 0;
    h->P[0] |= 1ull;
    pos = 1;
    for (int64_t k = 0; k < n; ++k) {
        while (top > 0 && (strict ? (A[stack[top - 1]] > A[k]) : (A[stack[top - 1]] >= A[k]))) {
            ++pos; /* closing parenthesis: bit stays 0 */
            --top;
        }
        stack[top++] = k;
        h->P[pos >> 6] |= 1ull << (pos & 63);
        ++pos;
    }
    pos += top + 1; /* closing parentheses for the stack and the root */
    free(stack);
    /* 2. rank directory */
    h->ones = (int64_t *)malloc(sizeof(int64_t) * (size_t)(h->nwords + 1));
    h->wmin = (int8_t *)malloc((size_t)h->nwords);
    h->wpos = (uint8_t *)malloc((size_t)h->nwords);
    if (!h->ones || !h->wmin || !h->wpos) {
        hrmq_port_free(h);
        return NULL;
    }
    h->ones[0] = 0;
    for (int64_t w = 0; w < h->nwords; ++w) h->ones[w + 1] = h->ones[w] + popc64(h->P[w]);
    /* 3. select samples */
    const int64_t total = h->ones[h->nwords];
    h->nsel = total / SEL_SAMPLE + 1;
    h->sel = (int64_t *)malloc(sizeof(int64_t) * (size_t)h->nsel);
    if (!h->sel) {
        hrmq_port_free(h);
        return NULL;
    }
    {
        int64_t s = 0, w = 0;
        for (int64_t k = 1; k <= total && s < h->nsel; k += SEL_SAMPLE, ++s) {
            while (h->ones[w + 1] < k) ++w;
            h->sel[s] = w << 6;
        }
        for (; s < h->nsel; ++s) h->sel[s] = (h->nwords - 1) << 6;
    }
    /* 4. per-word minima (relative) and the segment tree over absolute minima */
#pragma omp parallel for schedule(static)
    for (int64_t w = 0; w < h->nwords; ++w) {
        const uint64_t x = h->P[w];
        int e = 0, mn = 1 << 20, mp = 0;
        for (int byte = 0; byte < 8; ++byte) {
            const unsigned b = (unsigned)((x >> (8 * byte)) & 0xffu);
            if (e + T_MIN[b] <= mn) {
                mn = e + T_MIN[b];
                mp = 8 * byte + T_POS[b];
            }
            e += T_EXC[b];
        }
        h->wmin[w] = (int8_t)mn;
        h->wpos[w] = (uint8_t)mp;
    }
    h->tsize = 1;
    while (h->tsize < h->nwords) h->tsize <<= 1;
    h->tval = (int64_t *)malloc(sizeof(int64_t) * (size_t)(2 * h->tsize));
    h->tword = (int64_t *)malloc(sizeof(int64_t) * (size_t)(2 * h->tsize));
    if (!h->tval || !h->tword) {
        hrmq_port_free(h);
        return NULL;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < h->tsize; ++i) {
        if (i < h->nwords) {
            h->tval[h->tsize + i] = 2 * h->ones[i] - (i << 6) + h->wmin[i];
            h->tword[h->tsize + i] = i;
        } else {
            h->tval[h->tsize + i] = INT64_MAX;
            h->tword[h->tsize + i] = -1;
        }
    }
    for (int64_t i = h->tsize - 1; i >= 1; --i) {
        const int64_t a = h->tval[2 * i], b = h->tval[2 * i + 1];
        if (b <= a) { /* rightmost on ties */
            h->tval[i] = b;
            h->tword[i] = h->tword[2 * i + 1];
        } else {
            h->tval[i] = a;
            h->tword[i] = h->tword[2 * i];
        }
    }
    return h;
}

void hrmq_port_free(hrmq_port_t *h) {
    if (!h) return;
    free(h->P);
    free(h->ones);
    free(h->sel);
    free(h->wmin);
    free(h->wpos);
    free(h->tval);
    free(h->tword);
    free(h);
}

int64_t hrmq_port_bytes(const hrmq_port_t *h) {
    if (!h) return 0;
    return (int64_t)(h->nwords * (8 + 8 + 2) + h->nsel * 8 + 2 * h->tsize * 16);
}

int hrmq_port_query(const hrmq_port_t *h, const float *A, const int32_t *Q, int64_t q, float *val,
                    int32_t *idx, int nt) {
    if (!h || !Q || q < 0 || (!val && !idx)) return -1;
    if (nt > 0) omp_set_num_threads(nt);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < q; ++i) {
        const int64_t l = Q[2 * i], r = Q[2 * i + 1];
        const int64_t x = select1(h, l + 2), y = select1(h, r + 2);
        const int64_t k = rank1(h, rmq_excess(h, x, y)) - 2;
        if (idx) idx[i] = (int32_t)k;
        if (val) val[i] = A[k];
    }
    return 0;
}
