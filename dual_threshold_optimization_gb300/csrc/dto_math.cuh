// dto_math.cuh -- device arithmetic of the DTO engine.
//
// 1. The FP64 upper-tail specification P(X >= k), X ~ Hypergeometric(N, K, n),
//    as a fixed sequence of IEEE binary64 operations.  Every operation is an
//    explicitly rounded intrinsic (__dadd_rn, __dmul_rn, __fma_rn, __ddiv_rn),
//    so nvcc cannot contract or reorder it; the FP64 results are therefore a
//    deterministic function of (N, K, n, k) and the double-double log-factorial
//    table.  Replaces the statrs 0.17.1 call in
//    src/stat_operations/hypergeometric_pvalue.rs:40-49 of the reference.
// 2. Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) for the on-device
//    permutations.
#pragma once
#include <cstdint>

namespace dto {

// ---------------------------------------------------------------------------
// Double-double arithmetic (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2).
// ---------------------------------------------------------------------------
struct dd { double hi, lo; };

__device__ __forceinline__ dd two_sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double bb = __dsub_rn(s, a);
  double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dd fast_two_sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double e = __dsub_rn(b, __dsub_rn(s, a));
  return {s, e};
}
__device__ __forceinline__ dd dd_add(dd x, dd y) {
  dd s = two_sum(x.hi, y.hi);
  dd t = two_sum(x.lo, y.lo);
  double e = __dadd_rn(s.lo, t.hi);
  dd u = fast_two_sum(s.hi, e);
  e = __dadd_rn(u.lo, t.lo);
  return fast_two_sum(u.hi, e);
}
__device__ __forceinline__ dd dd_sub(dd x, dd y) { return dd_add(x, dd{-y.hi, -y.lo}); }

// ---------------------------------------------------------------------------
// e^L for a double-double L in [-746, 0]: reduction L = k ln2 + r by fma
// against ln 2 split in two doubles (Cody & Waite's method), the degree-14
// Taylor polynomial of e^r by Horner's rule, then scaling by 2^k.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pow2i(long long k) {  // 2^k, -1022 <= k <= 1023
  return __longlong_as_double((k + 1023LL) << 52);
}

__device__ __forceinline__ double exp_dd(dd L) {
  if (L.hi < -746.0) return 0.0;
  const double kLn2Hi = 0x1.62e42fefa39efp-1;   // ln 2 rounded to double
  const double kLn2Lo = 0x1.abc9e3b39803fp-56;  // ln 2 - kLn2Hi
  const double kInvLn2 = 0x1.71547652b82fep+0;  // 1 / ln 2 rounded
  double t = __dmul_rn(L.hi, kInvLn2);
  double kf = floor(__dadd_rn(t, 0.5));
  double r = __fma_rn(-kf, kLn2Hi, L.hi);
  r = __fma_rn(-kf, kLn2Lo, r);
  r = __dadd_rn(r, L.lo);
  // 1/j!, j = 0..14, each rounded to nearest double
  const double c0 = 1.0, c1 = 1.0, c2 = 0.5;
  const double c3 = 0x1.5555555555555p-3, c4 = 0x1.5555555555555p-5;
  const double c5 = 0x1.1111111111111p-7, c6 = 0x1.6c16c16c16c17p-10;
  const double c7 = 0x1.a01a01a01a01ap-13, c8 = 0x1.a01a01a01a01ap-16;
  const double c9 = 0x1.71de3a556c734p-19, c10 = 0x1.27e4fb7789f5cp-22;
  const double c11 = 0x1.ae64567f544e4p-26, c12 = 0x1.1eed8eff8d898p-29;
  const double c13 = 0x1.6124613a86d09p-33, c14 = 0x1.93974a8c07c9dp-37;
  double y = c14;
  y = __fma_rn(y, r, c13); y = __fma_rn(y, r, c12); y = __fma_rn(y, r, c11);
  y = __fma_rn(y, r, c10); y = __fma_rn(y, r, c9);  y = __fma_rn(y, r, c8);
  y = __fma_rn(y, r, c7);  y = __fma_rn(y, r, c6);  y = __fma_rn(y, r, c5);
  y = __fma_rn(y, r, c4);  y = __fma_rn(y, r, c3);  y = __fma_rn(y, r, c2);
  y = __fma_rn(y, r, c1);  y = __fma_rn(y, r, c0);
  long long k = (long long)kf;
  if (k >= -1021) return __dmul_rn(y, pow2i(k));
  return __dmul_rn(__dmul_rn(y, pow2i(k + 600)), pow2i(-600));
}

// ---------------------------------------------------------------------------
// ln pmf(k) of Hypergeometric(N, a, b) in double-double, a <= b, from the
// double-double log-factorial table lf[m] = ln(m!).  The parenthesisation is
// part of the specification.
// ---------------------------------------------------------------------------
__device__ __forceinline__ dd lfv(const double2* __restrict__ lf, long long m) {
  double2 v = __ldg(lf + m);
  return {v.x, v.y};
}

__device__ __forceinline__ dd logpmf_dd(const double2* __restrict__ lf, long long N, long long a,
                                        long long b, long long k) {
  dd num = dd_add(dd_add(lfv(lf, a), lfv(lf, N - a)), dd_add(lfv(lf, b), lfv(lf, N - b)));
  num = dd_sub(num, lfv(lf, N));
  dd den = dd_add(dd_add(lfv(lf, k), lfv(lf, a - k)), dd_add(lfv(lf, b - k), lfv(lf, N - a - b + k)));
  return dd_sub(num, den);
}

// P(X >= k).  k == 0 -> 1.0 (hypergeometric_pvalue.rs:44-46); (K, n) are
// canonicalised to (min, max) so the value is symmetric in them.  Above the
// mode m = floor((a+1)(b+1)/(N+2)) every ratio pmf(j+1)/pmf(j) is below 1 and
// decreasing: the tail is pmf(k) times the sum of ratio products, summed
// upward.  At or below the mode it is 1 - P(X <= k-1), the lower sum summed
// downward (ratios pmf(j-1)/pmf(j), also below 1 and decreasing).  Either sum
// stops at the support end or once the remainder bound t r / (1 - r) is at
// most 2^-54 of the sum.  The factors of each ratio are exact integers held
// in doubles (their products stay below 2^53).
static __device__ __noinline__ double sf64(const double2* __restrict__ lf, long long N, long long K,
                                           long long n, long long k) {
  if (k <= 0) return 1.0;
  long long a = K < n ? K : n;
  long long b = K < n ? n : K;
  long long lo = a + b - N;
  if (lo < 0) lo = 0;
  if (k > a) return 0.0;
  if (k <= lo) return 1.0;
  long long m = ((a + 1) * (b + 1)) / (N + 2);
  if (k > m) {
    double E = exp_dd(logpmf_dd(lf, N, a, b, k));
    double S = 1.0, t = 1.0;
    double aj = (double)(a - k), bj = (double)(b - k), j1 = (double)(k + 1), cj = (double)(N - a - b + k + 1);
    while (aj > 0.0) {
      double r = __ddiv_rn(__dmul_rn(aj, bj), __dmul_rn(j1, cj));
      t = __dmul_rn(t, r);
      S = __dadd_rn(S, t);
      aj = __dsub_rn(aj, 1.0); bj = __dsub_rn(bj, 1.0);
      j1 = __dadd_rn(j1, 1.0); cj = __dadd_rn(cj, 1.0);
      if (__dmul_rn(t, r) <= __dmul_rn(__dmul_rn(S, 0x1p-54), __dsub_rn(1.0, r))) break;
    }
    double p = __dmul_rn(E, S);
    return p > 1.0 ? 1.0 : p;
  } else {
    double E = exp_dd(logpmf_dd(lf, N, a, b, k - 1));
    double S = 1.0, t = 1.0;
    // j runs from k-1 down to lo+1: ratio j (c + j) / ((a - j + 1)(b - j + 1))
    double jd = (double)(k - 1), cj = (double)(N - a - b + k - 1);
    double aj = (double)(a - k + 2), bj = (double)(b - k + 2);
    const double lod = (double)lo;
    while (jd > lod) {
      double r = __ddiv_rn(__dmul_rn(jd, cj), __dmul_rn(aj, bj));
      t = __dmul_rn(t, r);
      S = __dadd_rn(S, t);
      jd = __dsub_rn(jd, 1.0); cj = __dsub_rn(cj, 1.0);
      aj = __dadd_rn(aj, 1.0); bj = __dadd_rn(bj, 1.0);
      if (__dmul_rn(t, r) <= __dmul_rn(__dmul_rn(S, 0x1p-54), __dsub_rn(1.0, r))) break;
    }
    double p = __dsub_rn(1.0, __dmul_rn(E, S));
    return p < 0.0 ? 0.0 : p;
  }
}

// Tie-break order of src/dto/optimize_main.rs:73-112: smaller p, then larger
// overlap, then smaller (rank1, rank2).  Thresholds increase with the grid
// index, so (i, j) order equals (rank1, rank2) order.
__device__ __forceinline__ bool better(double p, int k, int i, int j, double bp, int bk, int bi,
                                       int bj) {
  if (p != bp) return p < bp;
  if (k != bk) return k > bk;
  if (i != bi) return i < bi;
  return j < bj;
}

// ---------------------------------------------------------------------------
// Philox4x32-10.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

}  // namespace dto
