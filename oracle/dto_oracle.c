/*
 * dto_oracle.c -- CPU oracle for the Dual Threshold Optimization permutation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs
 * may load it.  The product library (dual_threshold_optimization_gb300) does not
 * link, import or call anything here.
 *
 * It restates, in plain C, the reference crate's algorithm for the hot path
 * (paths relative to the reference project):
 *   thresholds            src/collections/ranked.rs:359-375 (generate_thresholds,
 *                         including the quirk that the last threshold is NOT
 *                         clamped to the maximum rank: lines 370-372 edit the old
 *                         vector, which is then overwritten at line 374)
 *   stable sort by rank   src/collections/ranked.rs:527-542
 *   set by threshold      src/collections/ranked.rs:561-568,
 *                         src/collections/permuted.rs:90-101 (permuted view)
 *   pair loop             src/dto/process_threshold_pairs.rs:71-131
 *   intersection          src/stat_operations/intersect_genes.rs:38-56
 *   upper tail            src/stat_operations/hypergeometric_pvalue.rs:33-50
 *   argmin + tie-break    src/dto/optimize_main.rs:53-118
 *   empirical p-value     src/stat_operations/empirical_pvalue.rs:109-187
 *   FDR lower bound       src/stat_operations/fdr.rs:29-60
 *
 * The reference evaluates the hypergeometric tail with the third-party crate
 * statrs 0.17.1 (Cargo.lock), which is not vendored.  Its source is not used.
 * The tail here is restated from the mathematics as a fixed sequence of IEEE
 * binary64 operations (the "FP64 tail specification" below).  The CUDA kernels
 * implement the same specification independently, so both sides produce the
 * same bits; the tests additionally check this specification against mpmath
 * and against the reference's golden values.
 *
 * Build with -ffp-contract=off: every fused multiply-add is an explicit fma().
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* Double-double arithmetic (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2).         */
/* ------------------------------------------------------------------------- */
typedef struct { double hi, lo; } dd_t;

static inline dd_t two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    dd_t r = {s, e};
    return r;
}
static inline dd_t fast_two_sum(double a, double b) {
    double s = a + b;
    double e = b - (s - a);
    dd_t r = {s, e};
    return r;
}
static inline dd_t dd_add(dd_t x, dd_t y) {
    dd_t s = two_sum(x.hi, y.hi);
    dd_t t = two_sum(x.lo, y.lo);
    double e = s.lo + t.hi;
    dd_t u = fast_two_sum(s.hi, e);
    e = u.lo + t.lo;
    return fast_two_sum(u.hi, e);
}
static inline dd_t dd_neg(dd_t x) { dd_t r = {-x.hi, -x.lo}; return r; }
static inline dd_t dd_sub(dd_t x, dd_t y) { return dd_add(x, dd_neg(y)); }
static inline dd_t dd_mul(dd_t x, dd_t y) {
    double p = x.hi * y.hi;
    double e = fma(x.hi, y.hi, -p);
    e = fma(x.hi, y.lo, e);
    e = fma(x.lo, y.hi, e);
    return fast_two_sum(p, e);
}
/* x / d for an exactly representable integer d > 0. */
static inline dd_t dd_div_int(dd_t x, double d) {
    double q1 = x.hi / d;
    double r = fma(-q1, d, x.hi);
    r = r + x.lo;
    double q2 = r / d;
    return fast_two_sum(q1, q2);
}

/* ------------------------------------------------------------------------- */
/* Log-factorial table lf(m) = ln(m!) in double-double.                       */
/* Recurrence: ln(m) = ln(m-1) + 2*atanh(1/(2m-1)), since m/(m-1) equals       */
/* (1+s)/(1-s) with s = 1/(2m-1); atanh by its Taylor series s + s^3/3 + ...   */
/* summed until a term falls below 2^-110 of the partial sum.                  */
/* ------------------------------------------------------------------------- */
OR_EXPORT void or_lf_table(int64_t nmax, double* hi, double* lo) {
    dd_t lf = {0.0, 0.0};
    dd_t ln = {0.0, 0.0};
    hi[0] = 0.0; lo[0] = 0.0;
    if (nmax >= 1) { hi[1] = 0.0; lo[1] = 0.0; }
    for (int64_t m = 2; m <= nmax; ++m) {
        double d = (double)(2 * m - 1);
        dd_t one = {1.0, 0.0};
        dd_t s = dd_div_int(one, d);
        dd_t s2 = dd_mul(s, s);
        dd_t pw = s;
        dd_t sum = s;
        for (int64_t i = 1; i < 200; ++i) {
            pw = dd_mul(pw, s2);
            dd_t term = dd_div_int(pw, (double)(2 * i + 1));
            sum = dd_add(sum, term);
            if (fabs(term.hi) < ldexp(fabs(sum.hi), -110)) break;
        }
        dd_t two_sum_v = {2.0 * sum.hi, 2.0 * sum.lo};
        ln = dd_add(ln, two_sum_v);
        lf = dd_add(lf, ln);
        hi[m] = lf.hi;
        lo[m] = lf.lo;
    }
}

/* ------------------------------------------------------------------------- */
/* exp of a double-double argument, L in [-746, 0].                           */
/* Method: argument reduction L = k*ln2 + r (Cody & Waite 1980 style, with     */
/* the reduction done by fma against ln2 split into two doubles), then the     */
/* Taylor polynomial of e^r of degree 14 evaluated by Horner's rule, then      */
/* scaling by 2^k built from the exponent field.                               */
/* ------------------------------------------------------------------------- */
static const double OR_LN2_HI = 0x1.62e42fefa39efp-1;   /* ln 2 rounded to double */
static const double OR_LN2_LO = 0x1.abc9e3b39803fp-56;  /* ln 2 - OR_LN2_HI       */
static const double OR_INV_LN2 = 0x1.71547652b82fep+0;  /* 1/ln 2 rounded         */

static inline double pow2i(int64_t k) { /* 2^k for -1022 <= k <= 1023 */
    uint64_t bits = (uint64_t)(k + 1023) << 52;
    double r;
    memcpy(&r, &bits, 8);
    return r;
}

static double or_exp_dd(dd_t L) {
    if (L.hi < -746.0) return 0.0;
    double t = L.hi * OR_INV_LN2;
    double kf = floor(t + 0.5);
    double r = fma(-kf, OR_LN2_HI, L.hi);
    r = fma(-kf, OR_LN2_LO, r);
    r = r + L.lo;
    /* 1/j! for j = 14 .. 0 */
    static const double c[15] = {
        1.0, 1.0, 0.5, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0, 1.0 / 5040.0,
        1.0 / 40320.0, 1.0 / 362880.0, 1.0 / 3628800.0, 1.0 / 39916800.0,
        1.0 / 479001600.0, 1.0 / 6227020800.0, 1.0 / 87178291200.0};
    double y = c[14];
    for (int j = 13; j >= 0; --j) y = fma(y, r, c[j]);
    int64_t k = (int64_t)kf;
    if (k >= -1021) return y * pow2i(k);
    return (y * pow2i(k + 600)) * pow2i(-600);
}

/* ------------------------------------------------------------------------- */
/* FP64 tail specification: P(X >= k), X ~ Hypergeometric(N, K, n).           */
/* (K, n) are canonicalised to a = min, b = max so the value is symmetric.    */
/* Above the mode m = floor((a+1)(b+1)/(N+2)) every ratio pmf(j+1)/pmf(j) is  */
/* below 1 and decreasing, so P = pmf(k) * sum of ratio products, summed      */
/* upward; at or below the mode P = 1 - P(X <= k-1), the lower sum summed     */
/* downward (its ratios pmf(j-1)/pmf(j) are below 1 and decreasing too).      */
/* ------------------------------------------------------------------------- */
static inline dd_t LFV(const double* h, const double* l, int64_t m) {
    dd_t r = {h[m], l[m]};
    return r;
}

static dd_t or_logpmf_dd(const double* h, const double* l, int64_t N, int64_t a, int64_t b, int64_t k) {
    dd_t num = dd_add(dd_add(LFV(h, l, a), LFV(h, l, N - a)), dd_add(LFV(h, l, b), LFV(h, l, N - b)));
    num = dd_sub(num, LFV(h, l, N));
    dd_t den = dd_add(dd_add(LFV(h, l, k), LFV(h, l, a - k)), dd_add(LFV(h, l, b - k), LFV(h, l, N - a - b + k)));
    return dd_sub(num, den);
}

OR_EXPORT double or_sf64(const double* h, const double* l, int64_t N, int64_t K, int64_t n, int64_t k) {
    /* hypergeometric_pvalue.rs:44-46: k == 0 gives exactly 1.0 */
    if (k <= 0) return 1.0;
    int64_t a = K < n ? K : n;
    int64_t b = K < n ? n : K;
    int64_t lo = a + b - N;
    if (lo < 0) lo = 0;
    if (k > a) return 0.0;
    if (k <= lo) return 1.0;
    int64_t m = ((a + 1) * (b + 1)) / (N + 2);
    int64_t c = N - a - b;
    if (k > m) {
        double E = or_exp_dd(or_logpmf_dd(h, l, N, a, b, k));
        double S = 1.0, t = 1.0;
        int64_t j = k;
        while (j < a) {
            double num = (double)((a - j) * (b - j));
            double den = (double)((j + 1) * (c + j + 1));
            double r = num / den;
            t = t * r;
            S = S + t;
            j = j + 1;
            /* ratios decrease above the mode, so the remainder is at most
             * t r / (1 - r): stop once that is below 2^-54 of the sum */
            if (t * r <= (S * 0x1p-54) * (1.0 - r)) break;
        }
        double p = E * S;
        return p > 1.0 ? 1.0 : p;
    } else {
        double E = or_exp_dd(or_logpmf_dd(h, l, N, a, b, k - 1));
        double S = 1.0, t = 1.0;
        int64_t j = k - 1;
        while (j > lo) {
            double num = (double)(j * (c + j));
            double den = (double)((a - j + 1) * (b - j + 1));
            double r = num / den;
            t = t * r;
            S = S + t;
            j = j - 1;
            if (t * r <= (S * 0x1p-54) * (1.0 - r)) break;
        }
        double p = 1.0 - E * S;
        return p < 0.0 ? 0.0 : p;
    }
}

/* log of the pmf, rounded to double (used by tests for the screen bound). */
OR_EXPORT double or_logpmf(const double* h, const double* l, int64_t N, int64_t K, int64_t n, int64_t k) {
    int64_t a = K < n ? K : n;
    int64_t b = K < n ? n : K;
    dd_t L = or_logpmf_dd(h, l, N, a, b, k);
    return L.hi + L.lo;
}

/* ------------------------------------------------------------------------- */
/* Thresholds (ranked.rs:359-375).                                            */
/* ------------------------------------------------------------------------- */
OR_EXPORT int64_t or_thresholds(uint32_t max_rank, uint32_t* out, int64_t cap) {
    int64_t n = 0;
    uint32_t current = 1;
    while (current <= max_rank) {
        if (n < cap) out[n] = current;
        ++n;
        double nx = floor((double)current * 1.01 + 1.0);
        if (nx >= 4294967296.0) break;
        current = (uint32_t)nx;
    }
    /* ranked.rs:370-372 modify the previous threshold vector, which line 374
     * then replaces: the last threshold stays as generated. */
    return n;
}

/* Stable sort of (rank, item) by rank (ranked.rs:527-542): insertion into a
 * merge sort that keeps equal ranks in input order. */
static void msort(uint32_t* r, int32_t* f, uint32_t* tr, int32_t* tf, int64_t n) {
    if (n < 2) return;
    int64_t h = n / 2;
    msort(r, f, tr, tf, h);
    msort(r + h, f + h, tr, tf, n - h);
    int64_t i = 0, j = h, o = 0;
    while (i < h && j < n) {
        if (r[j] < r[i]) { tr[o] = r[j]; tf[o++] = f[j++]; }
        else { tr[o] = r[i]; tf[o++] = f[i++]; }
    }
    while (i < h) { tr[o] = r[i]; tf[o++] = f[i++]; }
    while (j < n) { tr[o] = r[j]; tf[o++] = f[j++]; }
    memcpy(r, tr, (size_t)n * 4);
    memcpy(f, tf, (size_t)n * 4);
}

OR_EXPORT void or_stable_sort(int64_t n, uint32_t* ranks, int32_t* items) {
    uint32_t* tr = (uint32_t*)malloc((size_t)(n > 0 ? n : 1) * 4);
    int32_t* tf = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * 4);
    msort(ranks, items, tr, tf, n);
    free(tr);
    free(tf);
}

/* ------------------------------------------------------------------------- */
/* Pair evaluation, histogram formulation.                                    */
/* Inputs: ranks sorted ascending; feat1/feat2 dense feature ids (>= 0) of the */
/* feature at each sorted position; idx1/idx2 the permuted views' index arrays */
/* (permuted.rs:34, shuffled indices into the sorted list) or NULL.  The set   */
/* for threshold t is {feat[idx[p]] : rank[p] <= t} (permuted.rs:90-101).      */
/* ------------------------------------------------------------------------- */
typedef struct {
    uint32_t rank1, rank2;
    int64_t set1_len, set2_len, intersection_size;
    double pvalue;
    int32_t i, j;
} or_record_t;

/* (p asc, k desc, rank1 asc, rank2 asc): optimize_main.rs:73-112 */
static int better(double p, int64_t k, uint32_t r1, uint32_t r2, const or_record_t* b) {
    if (p != b->pvalue) return p < b->pvalue;
    if (k != b->intersection_size) return k > b->intersection_size;
    if (r1 != b->rank1) return r1 < b->rank1;
    return r2 < b->rank2;
}

/* mode 0: histogram + 2D prefix; mode 1: literal per-cell intersection of
 * feature ids (intersect_genes.rs semantics, O(n1*n2*(N1+N2))). */
OR_EXPORT int or_optimize(const uint32_t* ranks1, const int32_t* feat1, int64_t N1,
                          const uint32_t* ranks2, const int32_t* feat2, int64_t N2,
                          int64_t nfeat, int64_t population,
                          const int32_t* idx1, const int32_t* idx2,
                          const double* lfh, const double* lfl, int mode,
                          or_record_t* best, or_record_t* all /* nullable [n1*n2] */) {
    if (N1 <= 0 || N2 <= 0) return -1;
    uint32_t max1 = ranks1[N1 - 1], max2 = ranks2[N2 - 1];
    int64_t n1 = or_thresholds(max1, NULL, 0), n2 = or_thresholds(max2, NULL, 0);
    if (n1 == 0 || n2 == 0) return -1;
    uint32_t* T1 = (uint32_t*)malloc((size_t)n1 * 4);
    uint32_t* T2 = (uint32_t*)malloc((size_t)n2 * 4);
    or_thresholds(max1, T1, n1);
    or_thresholds(max2, T2, n2);
    /* set sizes c(t) = #{rank <= t}: permutation independent */
    int64_t* c1 = (int64_t*)calloc((size_t)n1, 8);
    int64_t* c2 = (int64_t*)calloc((size_t)n2, 8);
    for (int64_t i = 0, p = 0; i < n1; ++i) { while (p < N1 && ranks1[p] <= T1[i]) ++p; c1[i] = p; }
    for (int64_t j = 0, p = 0; j < n2; ++j) { while (p < N2 && ranks2[p] <= T2[j]) ++p; c2[j] = p; }
    int rc = 0;
    best->pvalue = INFINITY;
    best->intersection_size = -1;
    best->rank1 = 0xffffffffu;
    best->rank2 = 0xffffffffu;
    if (mode == 0) {
        /* bin of each feature in each list (n = never) */
        int32_t* b1 = (int32_t*)malloc((size_t)nfeat * 4);
        int32_t* b2 = (int32_t*)malloc((size_t)nfeat * 4);
        for (int64_t f = 0; f < nfeat; ++f) { b1[f] = -1; b2[f] = -1; }
        for (int64_t p = 0, i = 0; p < N1; ++p) {
            while (i < n1 && T1[i] < ranks1[p]) ++i;
            int32_t g = feat1[idx1 ? idx1[p] : p];
            b1[g] = (i < n1) ? (int32_t)i : (int32_t)n1;
        }
        for (int64_t p = 0, j = 0; p < N2; ++p) {
            while (j < n2 && T2[j] < ranks2[p]) ++j;
            int32_t g = feat2[idx2 ? idx2[p] : p];
            b2[g] = (j < n2) ? (int32_t)j : (int32_t)n2;
        }
        int64_t* H = (int64_t*)calloc((size_t)(n1 * n2), 8);
        for (int64_t f = 0; f < nfeat; ++f)
            if (b1[f] >= 0 && b2[f] >= 0 && b1[f] < n1 && b2[f] < n2) H[b1[f] * n2 + b2[f]] += 1;
        for (int64_t i = 0; i < n1; ++i)
            for (int64_t j = 0; j < n2; ++j) {
                int64_t v = H[i * n2 + j];
                if (i > 0) v += H[(i - 1) * n2 + j];
                if (j > 0) v += H[i * n2 + j - 1];
                if (i > 0 && j > 0) v -= H[(i - 1) * n2 + j - 1];
                H[i * n2 + j] = v;
            }
        for (int64_t i = 0; i < n1; ++i)
            for (int64_t j = 0; j < n2; ++j) {
                int64_t k = H[i * n2 + j];
                double p = or_sf64(lfh, lfl, population, c1[i], c2[j], k);
                if (all) {
                    or_record_t* r = &all[i * n2 + j];
                    r->rank1 = T1[i]; r->rank2 = T2[j]; r->set1_len = c1[i]; r->set2_len = c2[j];
                    r->intersection_size = k; r->pvalue = p; r->i = (int32_t)i; r->j = (int32_t)j;
                }
                if (better(p, k, T1[i], T2[j], best)) {
                    best->pvalue = p; best->intersection_size = k; best->rank1 = T1[i]; best->rank2 = T2[j];
                    best->set1_len = c1[i]; best->set2_len = c2[j]; best->i = (int32_t)i; best->j = (int32_t)j;
                }
            }
        free(H); free(b1); free(b2);
    } else {
        /* literal: per cell, the set of list-1 feature ids and a count of the
         * list-2 set members that are in it (intersect_genes.rs:44-55). */
        uint8_t* inset = (uint8_t*)calloc((size_t)nfeat, 1);
        for (int64_t i = 0; i < n1; ++i) {
            for (int64_t j = 0; j < n2; ++j) {
                memset(inset, 0, (size_t)nfeat);
                for (int64_t p = 0; p < N1; ++p)
                    if (ranks1[p] <= T1[i]) inset[feat1[idx1 ? idx1[p] : p]] = 1;
                int64_t k = 0;
                for (int64_t p = 0; p < N2; ++p)
                    if (ranks2[p] <= T2[j]) k += inset[feat2[idx2 ? idx2[p] : p]];
                double p = or_sf64(lfh, lfl, population, c1[i], c2[j], k);
                if (all) {
                    or_record_t* r = &all[i * n2 + j];
                    r->rank1 = T1[i]; r->rank2 = T2[j]; r->set1_len = c1[i]; r->set2_len = c2[j];
                    r->intersection_size = k; r->pvalue = p; r->i = (int32_t)i; r->j = (int32_t)j;
                }
                if (better(p, k, T1[i], T2[j], best)) {
                    best->pvalue = p; best->intersection_size = k; best->rank1 = T1[i]; best->rank2 = T2[j];
                    best->set1_len = c1[i]; best->set2_len = c2[j]; best->i = (int32_t)i; best->j = (int32_t)j;
                }
            }
        }
        free(inset);
    }
    free(T1); free(T2); free(c1); free(c2);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* FDR lower bound (fdr.rs:29-60) and empirical p-value (empirical_pvalue.rs). */
/* ------------------------------------------------------------------------- */
OR_EXPORT double or_fdr(int64_t l1, int64_t l2, int64_t overlap, int64_t population, double sensitivity) {
    double df = (double)overlap / sensitivity;
    if (df < 0.0) df = 0.0;
    double bm = (double)l1 - df; if (bm < 0.0) bm = 0.0;
    double rm = (double)l2 - df; if (rm < 0.0) rm = 0.0;
    double num = bm * rm;
    double den = (double)population * (double)overlap;
    return den > 0.0 ? num / den : 0.0;
}

OR_EXPORT double or_empirical(double p_obs, const double* p_perm, int64_t n_perm) {
    if (n_perm <= 0) return 1.0;
    int64_t c = 0;
    for (int64_t i = 0; i < n_perm; ++i) c += (p_perm[i] <= p_obs);
    return (double)c / (double)n_perm;
}

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the permutation       */
/* specification used by the GPU's on-device permutations:                     */
/*   one level of Rao-Sandelius bucketing (4096 buckets, bucket = top 12 bits  */
/*   of one 16-bit half of a Philox word per element), elements in each bucket */
/*   kept in index order, then a Fisher-Yates shuffle of each bucket from its  */
/*   own Philox stream with Lemire's unbiased bounded integers.  The result is */
/*   an exactly uniform permutation.                                           */
/* ------------------------------------------------------------------------- */
OR_EXPORT void or_philox4x32_10(const uint32_t* ctr_in, const uint32_t* key_in, uint32_t* out) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define OR_NBUCKET 4096

typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int used;
} or_stream_t;

static uint32_t stream_next(or_stream_t* s) {
    if (s->used == 4) {
        or_philox4x32_10(s->ctr, s->key, s->buf);
        s->ctr[0] += 1;
        s->used = 0;
    }
    return s->buf[s->used++];
}

static uint32_t bounded(or_stream_t* s, uint32_t range) {
    uint32_t x = stream_next(s);
    uint64_t m = (uint64_t)x * range;
    uint32_t l = (uint32_t)m;
    if (l < range) {
        uint32_t thr = (uint32_t)(-range) % range;
        while (l < thr) {
            x = stream_next(s);
            m = (uint64_t)x * range;
            l = (uint32_t)m;
        }
    }
    return (uint32_t)(m >> 32);
}

/* The bucket of element e: the low (e even) or high (e odd) 16 bits of word
 * (e / 2) % 4 of the Philox block at counter (e / 8, perm, pair,
 * 0x10000000 | tag<<24), and of those 16 bits the top 12. */
static uint32_t bucket_of(const uint32_t w[4], int32_t e) {
    const uint32_t word = w[(e >> 1) & 3];
    return (e & 1) ? (word >> 20) : ((word >> 4) & 0xFFFu);
}

/* sigma[p] for p in [0, L): the index placed at position p.
 * Every element draws a bucket in [0, 4096) (bucket_of); elements are grouped
 * by bucket in increasing e.  Each bucket is then shuffled by the forward
 * Fisher-Yates pass (i = 1..sz-1: swap positions i and j, j uniform in
 * [0, i]) whose draws come from the bucket's own Philox stream (counter
 * (call, perm, pair, 0x20000000 | tag<<24 | bucket), the four words of each
 * call in order) by Lemire's multiply-shift with rejection.  Independent
 * uniform buckets followed by uniform shuffles of the buckets give an exactly
 * uniform permutation (one level of Rao-Sandelius). */
OR_EXPORT void or_shuffle(uint64_t seed, uint32_t pair_id, uint32_t perm_id, uint32_t list_tag, int32_t L, int32_t* sigma) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t* bucket = (uint32_t*)malloc((size_t)(L > 0 ? L : 1) * 4);
    int64_t* cnt = (int64_t*)calloc(OR_NBUCKET + 1, sizeof(int64_t));
    int64_t* fill = (int64_t*)malloc(OR_NBUCKET * sizeof(int64_t));
    for (int32_t e = 0; e < L; ++e) {
        uint32_t ctr[4] = {(uint32_t)e >> 3, perm_id, pair_id, 0x10000000u | (list_tag << 24)};
        uint32_t w[4];
        or_philox4x32_10(ctr, key, w);
        bucket[e] = bucket_of(w, e);
        cnt[bucket[e] + 1] += 1;
    }
    for (int b = 0; b < OR_NBUCKET; ++b) cnt[b + 1] += cnt[b];
    for (int b = 0; b < OR_NBUCKET; ++b) fill[b] = cnt[b];
    for (int32_t e = 0; e < L; ++e) sigma[fill[bucket[e]]++] = e;
    for (int b = 0; b < OR_NBUCKET; ++b) {
        int64_t s0 = cnt[b], sz = cnt[b + 1] - cnt[b];
        or_stream_t st;
        st.key[0] = key[0]; st.key[1] = key[1];
        st.ctr[0] = 0; st.ctr[1] = perm_id; st.ctr[2] = pair_id;
        st.ctr[3] = 0x20000000u | (list_tag << 24) | (uint32_t)b;
        st.used = 4;
        for (int64_t i = 1; i < sz; ++i) {
            const uint32_t j = bounded(&st, (uint32_t)(i + 1));
            int32_t tmp = sigma[s0 + i];
            sigma[s0 + i] = sigma[s0 + j];
            sigma[s0 + j] = tmp;
        }
    }
    free(bucket);
    free(cnt);
    free(fill);
}

/* ------------------------------------------------------------------------- */
/* Reference-algorithm CPU baseline: string features, one hash set of the      */
/* list-1 set per cell (intersect_genes.rs:44-55, Rust's HashSet<&str>, whose  */
/* default hasher is SipHash-1-3), list-2 sets cached per threshold            */
/* (process_threshold_pairs.rs:92-98), FP64 tail per cell, tasks chunked over  */
/* threads as in run/single_node.rs:95-133.                                    */
/* ------------------------------------------------------------------------- */
#define ROTL(x, b) (uint64_t)(((x) << (b)) | ((x) >> (64 - (b))))
#define SIPROUND                                                                 \
    do {                                                                         \
        v0 += v1; v1 = ROTL(v1, 13); v1 ^= v0; v0 = ROTL(v0, 32);                \
        v2 += v3; v3 = ROTL(v3, 16); v3 ^= v2;                                   \
        v0 += v3; v3 = ROTL(v3, 21); v3 ^= v0;                                   \
        v2 += v1; v1 = ROTL(v1, 17); v1 ^= v2; v2 = ROTL(v2, 32);                \
    } while (0)

/* SipHash-1-3 (Aumasson & Bernstein 2012; one compression, three finalisation rounds). */
static uint64_t siphash13(const uint8_t* in, size_t len, uint64_t k0, uint64_t k1) {
    uint64_t v0 = 0x736f6d6570736575ULL ^ k0, v1 = 0x646f72616e646f6dULL ^ k1;
    uint64_t v2 = 0x6c7967656e657261ULL ^ k0, v3 = 0x7465646279746573ULL ^ k1;
    uint64_t b = ((uint64_t)len) << 56;
    size_t end = len - (len % 8);
    for (size_t i = 0; i < end; i += 8) {
        uint64_t m = 0;
        for (int q = 0; q < 8; ++q) m |= (uint64_t)in[i + q] << (8 * q);
        v3 ^= m; SIPROUND; v0 ^= m;
    }
    for (size_t q = 0; q < len % 8; ++q) b |= (uint64_t)in[end + q] << (8 * q);
    v3 ^= b; SIPROUND; v0 ^= b;
    v2 ^= 0xff;
    SIPROUND; SIPROUND; SIPROUND;
    return v0 ^ v1 ^ v2 ^ v3;
}

typedef struct {
    const char** s;
    uint64_t* h;
    uint32_t* used;
    int64_t nused;
    uint32_t mask;
} strset_t;

static void strset_init(strset_t* t, int64_t cap) {
    uint32_t sz = 16;
    while (sz < 2 * cap) sz <<= 1;
    t->s = (const char**)calloc(sz, sizeof(char*));
    t->h = (uint64_t*)calloc(sz, 8);
    t->used = (uint32_t*)calloc(sz, 4);
    t->nused = 0;
    t->mask = sz - 1;
}
static void strset_clear(strset_t* t) {
    for (int64_t q = 0; q < t->nused; ++q) t->s[t->used[q]] = NULL;
    t->nused = 0;
}
static void strset_insert(strset_t* t, const char* s, uint64_t k0, uint64_t k1) {
    uint64_t h = siphash13((const uint8_t*)s, strlen(s), k0, k1);
    uint32_t i = (uint32_t)h & t->mask;
    while (t->s[i]) {
        if (t->h[i] == h && strcmp(t->s[i], s) == 0) return;
        i = (i + 1) & t->mask;
    }
    t->s[i] = s; t->h[i] = h;
    t->used[t->nused++] = i;
}
static int strset_has(const strset_t* t, const char* s, uint64_t k0, uint64_t k1) {
    uint64_t h = siphash13((const uint8_t*)s, strlen(s), k0, k1);
    uint32_t i = (uint32_t)h & t->mask;
    while (t->s[i]) {
        if (t->h[i] == h && strcmp(t->s[i], s) == 0) return 1;
        i = (i + 1) & t->mask;
    }
    return 0;
}

typedef struct {
    const char* const* g1; const uint32_t* r1; int64_t N1;
    const char* const* g2; const uint32_t* r2; int64_t N2;
    int64_t population;
    const double* lfh; const double* lfl;
    const int32_t* idx1s; const int32_t* idx2s; /* [n_tasks][N1], [n_tasks][N2] or NULL */
    int64_t row_stride; /* evaluate every row_stride-th list-1 threshold (sampling) */
    int64_t t0, t1;     /* task range of this worker */
    or_record_t* out;
    int64_t cells_done;
} ref_job_t;

static void* ref_worker(void* arg) {
    ref_job_t* J = (ref_job_t*)arg;
    int64_t n1 = or_thresholds(J->r1[J->N1 - 1], NULL, 0), n2 = or_thresholds(J->r2[J->N2 - 1], NULL, 0);
    uint32_t* T1 = (uint32_t*)malloc((size_t)n1 * 4);
    uint32_t* T2 = (uint32_t*)malloc((size_t)n2 * 4);
    or_thresholds(J->r1[J->N1 - 1], T1, n1);
    or_thresholds(J->r2[J->N2 - 1], T2, n2);
    const char** set1 = (const char**)malloc((size_t)J->N1 * sizeof(char*));
    strset_t hs;
    strset_init(&hs, J->N1);
    uint64_t k0 = 0x0706050403020100ULL, k1 = 0x0f0e0d0c0b0a0908ULL;
    J->cells_done = 0;
    for (int64_t task = J->t0; task < J->t1; ++task) {
        const int32_t* idx1 = J->idx1s ? J->idx1s + task * J->N1 : NULL;
        const int32_t* idx2 = J->idx2s ? J->idx2s + task * J->N2 : NULL;
        /* The list-2 set for T2[j] is the permuted features at the sorted
         * positions p < c2(T2[j]); iterating that prefix visits the same
         * vector the reference caches per threshold. */
        or_record_t best;
        best.pvalue = INFINITY; best.intersection_size = -1; best.rank1 = best.rank2 = 0xffffffffu;
        for (int64_t i = 0; i < n1; i += J->row_stride) {
            int64_t s1 = 0;
            for (int64_t p = 0; p < J->N1; ++p)
                if (J->r1[p] <= T1[i]) set1[s1++] = J->g1[idx1 ? idx1[p] : p];
            for (int64_t j = 0; j < n2; ++j) {
                /* set2 for T2[j]: positions with rank <= T2[j] */
                int64_t s2 = 0;
                strset_clear(&hs);
                for (int64_t q = 0; q < s1; ++q) strset_insert(&hs, set1[q], k0, k1);
                int64_t k = 0;
                for (int64_t p = 0; p < J->N2 && J->r2[p] <= T2[j]; ++p) {
                    ++s2;
                    k += strset_has(&hs, J->g2[idx2 ? idx2[p] : p], k0, k1);
                }
                double pv = or_sf64(J->lfh, J->lfl, J->population, s1, s2, k);
                if (better(pv, k, T1[i], T2[j], &best)) {
                    best.pvalue = pv; best.intersection_size = k; best.rank1 = T1[i]; best.rank2 = T2[j];
                    best.set1_len = s1; best.set2_len = s2; best.i = (int32_t)i; best.j = (int32_t)j;
                }
                J->cells_done += 1;
            }
        }
        if (J->out) J->out[task] = best;
    }
    strset_clear(&hs);
    free(hs.s); free(hs.h); free(hs.used); free(set1); free(T1); free(T2);
    return NULL;
}

/* Runs n_tasks tasks over nthreads threads, chunked as ceil(n_tasks/nthreads)
 * (single_node.rs:95-98).  Returns the number of grid cells evaluated. */
OR_EXPORT int64_t or_ref_run(const char* const* g1, const uint32_t* r1, int64_t N1,
                             const char* const* g2, const uint32_t* r2, int64_t N2,
                             int64_t population, const double* lfh, const double* lfl,
                             const int32_t* idx1s, const int32_t* idx2s, int64_t n_tasks,
                             int64_t row_stride, int nthreads, or_record_t* out) {
    if (nthreads < 1) nthreads = 1;
    if (row_stride < 1) row_stride = 1;
    int64_t chunk = (n_tasks + nthreads - 1) / nthreads;
    if (chunk < 1) chunk = 1;
    int nj = (int)((n_tasks + chunk - 1) / chunk);
    pthread_t* th = (pthread_t*)malloc((size_t)(nj > 0 ? nj : 1) * sizeof(pthread_t));
    ref_job_t* jobs = (ref_job_t*)calloc((size_t)(nj > 0 ? nj : 1), sizeof(ref_job_t));
    for (int t = 0; t < nj; ++t) {
        ref_job_t* J = &jobs[t];
        J->g1 = g1; J->r1 = r1; J->N1 = N1; J->g2 = g2; J->r2 = r2; J->N2 = N2;
        J->population = population; J->lfh = lfh; J->lfl = lfl;
        J->idx1s = idx1s; J->idx2s = idx2s; J->row_stride = row_stride;
        J->t0 = t * chunk; J->t1 = (t + 1) * chunk < n_tasks ? (t + 1) * chunk : n_tasks;
        J->out = out;
        pthread_create(&th[t], NULL, ref_worker, J);
    }
    int64_t cells = 0;
    for (int t = 0; t < nj; ++t) { pthread_join(th[t], NULL); cells += jobs[t].cells_done; }
    free(th); free(jobs);
    return cells;
}
