// dto_grid.cuh -- the threshold-pair search of one task per warp.
//
// Replaces src/dto/process_threshold_pairs.rs:71-131 (the n1 x n2 loop with a
// set intersection and a hypergeometric tail per cell) and the argmin of
// src/dto/optimize_main.rs:53-118.
//
// Formulation.  A task is given as X[p], the label of the list-2 threshold
// column of the feature at list-1 position p (-1 if that feature never enters
// a list-2 set).  Row i of the grid holds the list-1 positions
// [rowstart[i], rowstart[i+1]) -- those whose rank lies in (T1[i-1], T1[i]].
// The warp sweeps the rows in order and keeps cnt[j] = #{features with list-1
// row <= i and list-2 column j} in shared memory; the overlap of cell (i, j)
// is the inclusive prefix sum of cnt over columns <= j, computed per row by
// each lane over its C consecutive columns plus a warp shuffle scan.  Counts
// are int32 and exact.
//
// Precision modes.
//   kModeFull64   every cell's FP64 tail (sf64); the plain FP64 path.
//   kModeScreen   three stages over a two-pass sweep.
//                 Stage 1 (every cell): a 32-bit fixed-point lower bound LB of
//                 ln p.  Pass A keeps each lane's smallest-LB cell; stage 2 on
//                 those 32 cells gives an upper bound B on the minimum ln p.
//                 Pass B sends every cell with LB <= B (+ slack) to a per-warp
//                 buffer; stage 2 (FP32 tail sum with a proven error bound)
//                 turns each into an interval [lo, hi] of ln p, tightens B to
//                 the smallest hi, and keeps the cells with lo <= B as
//                 survivors.  Stage 3 evaluates the survivors' FP64 tails and
//                 takes the argmin with the reference's tie-break.  The FP64
//                 argmin over the survivors is the FP64 argmin over all cells
//                 (argument at pass B below).
//   kModeDump     one task: every cell's overlap and FP64 p (debug export).
//
// The 32-bit screen.  ln pmf(k) = ln K! + ln (N-K)! + ln n! + ln (N-n)! - ln N!
//   - ln k! - ln (K-k)! - ln (n-k)! - ln (N-K-n+k)!, from the table
//   F[m] = round(ln(m!) * 2^f) held modulo 2^32 in shared memory.  The nine-term
//   integer sum is exact, so |LB/2^f - ln pmf| <= 9 * 0.5 * 2^-f.  Because
//   pmf(kk) <= P(X >= k) for every kk >= k, the bound is evaluated at
//   kk = max(k, m~) with m~ = round(K n / N), which keeps it tight for cells at
//   or below the mean (m~ lies in the support for any rounding of K n / N).
#pragma once
#include "dto_internal.h"
#include "dto_math.cuh"

namespace dto {

constexpr unsigned kFull = 0xffffffffu;

struct Best {
  double p;
  int k, i, j;
};

__device__ __forceinline__ Best best_init() { return Best{__longlong_as_double(0x7ff0000000000000LL), -1, 0x7fffffff, 0x7fffffff}; }

__device__ __forceinline__ void best_take(Best& b, double p, int k, int i, int j) {
  if (better(p, k, i, j, b.p, b.k, b.i, b.j)) b = Best{p, k, i, j};
}

__device__ __forceinline__ void warp_best(Best& b) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    double p = __shfl_xor_sync(kFull, b.p, d);
    int k = __shfl_xor_sync(kFull, b.k, d);
    int i = __shfl_xor_sync(kFull, b.i, d);
    int j = __shfl_xor_sync(kFull, b.j, d);
    best_take(b, p, k, i, j);
  }
}

__device__ __forceinline__ int lb_fix(const uint32_t* F, int K, int NK, uint32_t Arow, float Kf, int n,
                                      uint32_t Bcol, float qn, int k) {
  float mf = __fmaf_rn(Kf, qn, 12582912.0f);  // 1.5 * 2^23: round to nearest integer
  int m = __float_as_int(mf) - 0x4B400000;
  int kk = max(k, m);
  uint32_t s = Arow + Bcol - F[kk] - F[K - kk] - F[n - kk] - F[NK - n + kk];
  return (int)s;
}

// ln pmf(k) of cell (K, n, k) in fixed point, exact up to the table rounding.
__device__ __forceinline__ int logpmf_fix(const uint32_t* F, int N, uint32_t FN, int K, int n, int k) {
  uint32_t s = F[K] + F[N - K] - FN + F[n] + F[N - n] - F[k] - F[K - k] - F[n - k] - F[N - K - n + k];
  return (int)s;
}

// FP32 sum S = sum_j pmf(k+j)/pmf(k) from k >= mode (ratios below 1 and
// decreasing), stopped when the remainder bound t r / (1 - r) is below 2^-26 of
// the sum.  Each ratio carries <= 2^-24 (numerator) + 2^-24 (denominator) +
// 2^-22 (__fdividef) relative error and each product/sum <= 2^-24, so after d
// terms |S32/S - 1| <= d * 5e-7 to first order; __logf adds <= 1e-5 absolute
// for S below 4e8.  The bound used is d * 1e-6 + 2e-5 (twice that).
// Returns false if the sum did not settle within 8192 terms.
__device__ __forceinline__ bool tail32(int N, int a, int b, int k, float& logS, float& err) {
  float aj = (float)(a - k), bj = (float)(b - k), j1 = (float)(k + 1), cj = (float)(N - a - b + k + 1);
  float t = 1.f, S = 1.f;
  int d = 0;
  bool ok = false;
  for (; d < 8192; ++d) {
    if (aj <= 0.f) {
      ok = true;
      break;
    }
    float r = __fdividef(aj * bj, j1 * cj);
    t *= r;
    S += t;
    aj -= 1.f;
    bj -= 1.f;
    j1 += 1.f;
    cj += 1.f;
    if (t * r <= S * 0x1p-26f * (1.f - r)) {
      ok = true;
      ++d;
      break;
    }
  }
  logS = __logf(S);
  err = (float)d * 1e-6f + 2e-5f;
  return ok;
}

// Stage 2: fixed-point bounds lo <= 2^f ln P(X >= k) <= hi for one cell.
struct Interval {
  int lo, hi;
};

__device__ __forceinline__ Interval eval32(const uint32_t* F, int N, uint32_t FN, int K, int n, int k,
                                           double scale) {
  const int a = min(K, n), b = max(K, n);
  const long long mode = ((long long)(a + 1) * (long long)(b + 1)) / (long long)(N + 2);
  if (k <= 0) return Interval{-8, 8};  // p = 1
  // At or below the mode, P(X >= k) >= P(X >= mode), whose upper sum starts
  // where the ratios drop below 1; the upper bound is p <= 1.
  const bool below = (long long)k <= mode;
  const int k0 = below ? (int)mode : k;
  const int Lk = logpmf_fix(F, N, FN, K, n, k0);
  float logS, err;
  if (!tail32(N, a, b, k0, logS, err)) return Interval{Lk - kScreenSlack, kScreenSlack};
  const int lo = Lk - kScreenSlack + (int)floor((double)(logS - err) * scale) - 1;
  if (below) return Interval{min(lo, 0), kScreenSlack};
  const int hi = Lk + kScreenSlack + (int)ceil((double)(logS + err) * scale) + 1;
  return Interval{lo, min(hi, kScreenSlack)};
}

constexpr int kTableW = 48;  // pmf terms of the partial-sum lower bound

// FP32 partial sum of w terms from k (ratios below 1 from the mode up); the
// same error analysis as tail32 bounds |ln S32 - ln S| by d 1e-6 + 2e-5.
__device__ __forceinline__ float partial32(int N, int a, int b, int k, float& err) {
  float aj = (float)(a - k), bj = (float)(b - k), j1 = (float)(k + 1), cj = (float)(N - a - b + k + 1);
  float t = 1.f, S = 1.f;
  int d = 0;
#pragma unroll 4
  for (; d < kTableW - 1; ++d) {
    if (aj <= 0.f) break;
    float r = __fdividef(aj * bj, j1 * cj);
    t *= r;
    S += t;
    aj -= 1.f;
    bj -= 1.f;
    j1 += 1.f;
    cj += 1.f;
  }
  err = (float)d * 1e-6f + 2e-5f;
  return __logf(S);
}

// Fixed-point lower bound of ln P(X >= k) used to build the table.
__device__ __forceinline__ int lbt_fix(const uint32_t* __restrict__ F, int N, uint32_t FN, int K, int n,
                                       int k, long long mode, double scale) {
  const int a = min(K, n), b = max(K, n);
  const int k0 = (long long)k <= mode ? (int)mode : k;
  const int L = logpmf_fix(F, N, FN, K, n, k0);
  float err;
  float ls = partial32(N, a, b, k0, err);
  return L - kScreenSlack + (int)floor((double)(ls - err) * scale) - 1;
}

// Closed-form lower bound of ln P(X >= k), fixed point, for the stage-2 gate.
// With k0 = max(k, mode) and the pmf ratios r_x = pmf(x+1)/pmf(x)
// non-increasing (the hypergeometric pmf is log-concave),
//   P(X >= k) >= P(X >= k0) >= pmf(k0) sum_{j<w} rho^j = pmf(k0) (1 - rho^w) / (1 - rho)
// for any w <= a - k0 + 1, rho = r_{k0+w-2} (every ratio of the first w - 1
// terms is >= rho).  1 - rho = D / ((x+1)(N-a-b+x+1)) with the exact integer
// D = (N+2)(x+1) - (a+1)(b+1), x = k0 + w - 2, so there is no cancellation;
// the sum is -expm1(w log1p(-u)) / u, u = 1 - rho, each step a few ulps in
// FP32, far inside the 1e-4 nats subtracted.  The best of w = 4, 32, 256 is
// taken: a few transcendental operations instead of the 48 pmf terms of
// lbt_fix, and close to ln p for cells with a wide distribution, whose tails
// run to hundreds of terms.
__device__ __forceinline__ int lbg_fix(const uint32_t* F, int N, uint32_t FN, int K, int n, int k,
                                       long long mode, double scale) {
  const int a = min(K, n), b = max(K, n);
  const int k0 = (long long)k <= mode ? (int)mode : k;
  const int L = logpmf_fix(F, N, FN, K, n, k0);
  const long long ab1 = (long long)(a + 1) * (long long)(b + 1);
  float g = 0.f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int w = min(q == 0 ? 4 : q == 1 ? 32 : 256, a - k0 + 1);
    if (w < 2) break;
    const int x = k0 + w - 2;
    const long long D = (long long)(N + 2) * (long long)(x + 1) - ab1;
    float G = (float)w;
    if (D > 0) {
      const float u = __fdiv_rn((float)D, (float)(x + 1) * (float)(N - a - b + x + 1));
      G = -expm1f((float)w * log1pf(-fminf(u, 1.f))) / u;
    }
    g = fmaxf(g, logf(G));
  }
  return L - kScreenSlack + (int)floor((double)(g - 1e-4f) * scale) - 1;
}

// Stage 2 behind cheaper filters: a cell whose closed-form or partial-sum
// lower bound already exceeds B + 1 can neither be the FP64 argmin (its ln p
// is above B) nor lower B, so its tail is not summed.
__device__ __forceinline__ Interval eval32_filtered(const uint32_t* F, int N, uint32_t FN, int K, int n, int k,
                                                    double scale, int B) {
  const int a = min(K, n), b = max(K, n);
  const long long mode = ((long long)(a + 1) * (long long)(b + 1)) / (long long)(N + 2);
  if (k > 0) {
    if (lbg_fix(F, N, FN, K, n, k, mode, scale) > B + 1) return Interval{0x7fffffff, 0x7fffffff};
    if (lbt_fix(F, N, FN, K, n, k, mode, scale) > B + 1) return Interval{0x7fffffff, 0x7fffffff};
  }
  return eval32(F, N, FN, K, n, k, scale);
}

// Device-side guess of the task's bound B from the tasks already finished in
// this launch: a histogram of their final B in quarter-nat bins of -ln p.
// A guess is used only as a starting point: the sweep it starts is accepted
// only if some cell's upper bound reaches it (see the claim in the kernel).
constexpr int kNoGuess = 0x7fffffff;
constexpr int kGuessBins = 256;      // bin q holds -ln p in [q/4, (q+1)/4) nats
constexpr int kGuessMinTasks = 256;  // finished tasks before the guess is used

__device__ __forceinline__ void bound_record(unsigned* hist, int B, double scale) {
  double nats = -(double)B / scale;
  int q = (int)floor(nats * 4.0);
  q = max(0, min(kGuessBins - 1, q));
  atomicAdd(hist + q, 1u);
  atomicAdd(hist + kGuessBins, 1u);
}

// The bound below which 90% of the recorded tasks fell (lower edge of the
// bin that reaches 10% of the tasks counted from small -ln p), as fixed point.
__device__ __forceinline__ int bound_guess_bin(const unsigned* hist, int lane) {
  unsigned total = *((volatile const unsigned*)(hist + kGuessBins));
  if (total < kGuessMinTasks) return -1;
  unsigned want = total / 10;
  unsigned run = 0;
  int found = -1;
  for (int q0 = 0; q0 < kGuessBins; q0 += 32) {
    unsigned v = *((volatile const unsigned*)(hist + q0 + lane));
    unsigned incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    unsigned m = __ballot_sync(0xffffffffu, run + incl > want);
    if (m) {
      found = q0 + __ffs(m) - 1;
      break;
    }
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  return found;
}

// One pass over the rows.  fn(i, O, excl) is called once per row with the
// lane's per-column inclusive partial sums O[t] and the lane's exclusive
// offset; the overlap of cell (i, lane*C + t) is O[t] + excl.
template <int C, class RowFn>
__device__ __forceinline__ void sweep(const int16_t* __restrict__ x, const int* __restrict__ sRow, int n1,
                                      int* cnt, int lane, bool hwlab, RowFn&& fn) {
  constexpr int Cp = C | 1;
  // a label's counter: the label itself, or for the table sweep's form its
  // column's (hwlab: the tasks a table run left)
  auto slot = [&](int v) { return hwlab ? grid_label_of_column(column_of_hw_label(v, C), C) : v; };
  for (int q = lane; q < 32 * Cp; q += 32) cnt[q] = 0;
  __syncwarp();
  int s = sRow[0], e = sRow[1];
  int pre = (s + lane < e) ? (int)__ldg(x + s + lane) : -1;
  for (int i = 0; i < n1; ++i) {
    int cur = pre;
    int sN = e;
    int eN = (i + 2 <= n1) ? sRow[i + 2] : e;
    pre = (sN + lane < eN) ? (int)__ldg(x + sN + lane) : -1;
    if (cur >= 0) atomicAdd(&cnt[slot(cur)], 1);
    for (int p = s + 32 + lane; p < e; p += 32) {
      int v = __ldg(x + p);
      if (v >= 0) atomicAdd(&cnt[slot(v)], 1);
    }
    __syncwarp();
    int O[C];
    int run = 0;
#pragma unroll
    for (int t = 0; t < C; ++t) {
      run += cnt[lane * Cp + t];
      O[t] = run;
    }
    int incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += y;
    }
    __syncwarp();
    fn(i, O, incl - run);
    s = sN;
    e = eN;
  }
}

template <int C>
__global__ void __launch_bounds__(kGridWarps * 32, 1) grid_kernel(const GridArgs A) {
  constexpr int kCntInts = grid_cnt_ints(C);
  constexpr int kWarpInts = grid_warp_ints(C);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // an empty task list (the usual fallback list): nothing to load or sweep
  if (A.ntask_dev && *((volatile const int*)A.ntask_dev) == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n1 = A.P.n1, n2 = A.P.n2;
  const long long Npop = A.P.Npop;
  const int N = (int)Npop;

  uint32_t* sF = reinterpret_cast<uint32_t*>(smem_raw);
  const int fWords = A.smemF ? ((N + 1 + 3) & ~3) : 0;
  int* sRow = reinterpret_cast<int*>(sF + fWords);
  int* sWarp = sRow + ((n1 + 1 + 3) & ~3);
  int* cnt = sWarp + warp * kWarpInts;
  int2* cand = reinterpret_cast<int2*>(cnt + kCntInts);
  int* survCell = cnt + kCntInts + 2 * kCandCap;  // survivors: packed cell, overlap, lo
  int* survK = survCell + kSurvCap;
  int* survLo = survK + kSurvCap;

  if (A.smemF)
    for (int q = threadIdx.x; q <= N; q += blockDim.x) sF[q] = __ldg(A.P.F + q);
  for (int q = threadIdx.x; q <= n1; q += blockDim.x) sRow[q] = __ldg(A.P.rowstart + q);
  __syncthreads();
  const uint32_t* F = A.smemF ? sF : A.P.F;
  const double2* LF = A.P.LF;

  // Per-lane constants of the lane's columns j = lane*C + t.  Columns past n2
  // get n = N, which keeps every table index of the screen in range.
  int ncol[C];
  uint32_t Bc[C];
  float qc[C];
  const float invN = 1.0f / (float)N;
  const int tvalid = max(0, min(C, n2 - lane * C));
#pragma unroll
  for (int t = 0; t < C; ++t) {
    int j = lane * C + t;
    int n = (j < n2) ? __ldg(A.P.ncnt + j) : N;
    ncol[t] = n;
    Bc[t] = F[n] + F[N - n];
    qc[t] = (float)n * invN;
  }
  const uint32_t FN = F[N];
  unsigned long long n32 = 0, n64 = 0, nfall = 0;  // stage-2, FP64 evaluations, fallbacks

  // Cooperative screen: the CTA's warps share one task.  Every warp sweeps
  // all rows (the counters need every label) but evaluates only the cells of
  // rows i with i % kGridWarps == warp, and the bound B is shared through
  // shared memory; the warps' optima are reduced at the end.  This cuts the
  // latency of hard tasks (a flat landscape sends most cells to stage 2).
  static_assert(kGridWarps <= 32, "one lane per warp in the cooperative reduction");
  const bool coop = A.coop != 0 && A.mode == kModeScreen;
  __shared__ int sTask, sB;
  __shared__ double sBestP[kGridWarps];
  __shared__ int sBestK[kGridWarps], sBestI[kGridWarps], sBestJ[kGridWarps];
  const int ntask = A.ntask_dev ? *((volatile const int*)A.ntask_dev) : A.ntask;
  for (;;) {
    int b = 0;
    if (coop) {
      __syncthreads();  // the previous task is finished by every warp
      if (threadIdx.x == 0) {
        sTask = atomicAdd(A.work, 1);
        sB = kScreenSlack;
      }
      __syncthreads();
      b = sTask;
    } else {
      if (lane == 0) b = atomicAdd(A.work, 1);
      b = __shfl_sync(kFull, b, 0);
    }
    if (b >= ntask) break;
    if (A.task_list) b = A.task_list[b];
    const int16_t* x = A.X + (long long)b * A.xstride;
    auto my_row = [&](int i) { return !coop || i % kGridWarps == warp; };

    if (A.mode == kModeFull64 || A.mode == kModeDump) {
      Best best = best_init();
      sweep<C>(x, sRow, n1, cnt, lane, A.hwlab != 0, [&](int i, const int (&O)[C], int excl) {
        const int K = sRow[i + 1];
#pragma unroll
        for (int t = 0; t < C; ++t) {
          if (t < tvalid) {
            int k = O[t] + excl;
            int j = lane * C + t;
            double p = sf64(LF, Npop, K, ncol[t], k);
            if (A.mode == kModeDump) {
              A.dump_k[(long long)i * n2 + j] = k;
              A.dump_p[(long long)i * n2 + j] = p;
            }
            best_take(best, p, k, i, j);
          }
        }
      });
      n64 += (unsigned long long)n1 * (unsigned long long)tvalid;
      warp_best(best);
      if (lane == 0) A.out[b] = TaskResult{best.p, best.i, best.j, best.k, A.route};
      continue;
    }

    // ---- kModeScreen ----
    const double scale = ldexp(1.0, A.P.fshift);
    const int Bfloor = (int)floor(-700.0 * scale);  // keep cells whose FP64 p may underflow
    int B = kScreenSlack;       // running bound on the smallest ln p (fixed point)
    bool B_valid = false;       // B is attained by an evaluated cell
    int ncand = 0, nsurv = 0;
    Best best64 = best_init();

    // Stage 3: FP64 tails of the survivors that the current B admits.
    auto refine_survivors = [&]() {
      __syncwarp();
      Best lb = best64;
      int done = 0;
      for (int q = lane; q < nsurv; q += 32) {
        if (survLo[q] <= B + 1) {
          int ci = survCell[q] >> 16, cj = survCell[q] & 0xffff;
          double p = sf64(LF, Npop, sRow[ci + 1], __ldg(A.P.ncnt + cj), survK[q]);
          best_take(lb, p, survK[q], ci, cj);
          ++done;
        }
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) done += __shfl_xor_sync(kFull, done, d);
      n64 += (unsigned long long)done;
      warp_best(lb);
      best64 = lb;
      nsurv = 0;
      __syncwarp();
    };
    // Drop the survivors that the current B excludes.
    auto compact = [&]() {
      __syncwarp();
      int kept = 0;
      for (int r0 = 0; r0 < nsurv; r0 += 32) {
        int r = r0 + lane;
        int sc = 0, sk = 0, sl = 0;
        if (r < nsurv) { sc = survCell[r]; sk = survK[r]; sl = survLo[r]; }
        bool st = r < nsurv && sl <= B + 1;
        unsigned sm = __ballot_sync(kFull, st);
        __syncwarp();
        if (st) {
          int pos = kept + __popc(sm & ((1u << lane) - 1u));
          survCell[pos] = sc; survK[pos] = sk; survLo[pos] = sl;
        }
        kept += __popc(sm);
        __syncwarp();
      }
      nsurv = kept;
    };
    // Stage 2 on the candidate buffer: tighten B to the smallest upper bound,
    // keep the cells whose lower bound is within B.
    auto flush = [&]() {
      __syncwarp();
      for (int q0 = 0; q0 < ncand; q0 += 32) {
        int q = q0 + lane;
        Interval iv{0x7fffffff, 0x7fffffff};
        int2 c = make_int2(0, 0);
        if (q < ncand) {
          c = cand[q];
          int ci = c.x >> 16, cj = c.x & 0xffff;
          iv = eval32_filtered(F, N, FN, sRow[ci + 1], __ldg(A.P.ncnt + cj), c.y, scale, B);
        }
        int h = iv.hi;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) h = min(h, __shfl_xor_sync(kFull, h, d));
        if (h <= B) {
          B = max(h, Bfloor);
          B_valid = true;
        }
        if (coop) {
          // any warp's bound is attained by a cell of this task: take the least
          if (lane == 0) atomicMin(&sB, B);
          B = min(B, *((volatile int*)&sB));
        }
        bool keep = (q < ncand) && iv.lo <= B + 1;
        unsigned m = __ballot_sync(kFull, keep);
        int nk = __popc(m);
        if (nsurv + nk > kSurvCap) {
          compact();
          if (nsurv + nk > kSurvCap) refine_survivors();
        }
        if (keep) {
          int pos = nsurv + __popc(m & ((1u << lane) - 1u));
          survCell[pos] = c.x;
          survK[pos] = c.y;
          survLo[pos] = iv.lo;
        }
        nsurv += nk;
        __syncwarp();
      }
      n32 += (unsigned long long)ncand;
      ncand = 0;
      __syncwarp();
    };
    // One sweep: cells with LB <= B + slack go to stage 2 (B only decreases).
    auto candidate_sweep = [&]() {
      sweep<C>(x, sRow, n1, cnt, lane, A.hwlab != 0, [&](int i, const int (&O)[C], int excl) {
        if (!my_row(i)) return;
        const int K = sRow[i + 1];
        const int NK = N - K;
        const uint32_t Arow = F[K] + F[NK] - FN;
        const float Kf = (float)K;
        const int tau = B + kScreenSlack + 1;
        unsigned hit = 0;
#pragma unroll
        for (int t = 0; t < C; ++t) {
          int k = O[t] + excl;
          int lb = lb_fix(F, K, NK, Arow, Kf, ncol[t], Bc[t], qc[t], k);
          hit |= (t < tvalid && lb <= tau) ? (1u << t) : 0u;
        }
        while (__any_sync(kFull, hit != 0)) {
          // append to the buffer in (lane, column) order
          int cntHit = __popc(hit);
          int incl = cntHit;
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += y;
          }
          int total = __shfl_sync(kFull, incl, 31);
          int room = kCandCap - ncand;
          int pos = ncand + incl - cntHit;
#pragma unroll
          for (int t = 0; t < C; ++t) {
            if (hit & (1u << t)) {
              if (pos < kCandCap) {
                cand[pos] = make_int2((i << 16) | (lane * C + t), O[t] + excl);
                hit &= ~(1u << t);
              }
              ++pos;
            }
          }
          ncand += min(total, room);
          if (ncand >= kCandCap - 32 || __any_sync(kFull, hit != 0)) flush();
        }
      });
      flush();
    };

    // Claim: after a sweep that started with bound B0 and ended with a valid
    // B <= B0, the FP64 argmin c* (and every cell tied with it) is a survivor.
    // B is attained by a cell c_b with ln p_true(c_b) <= B 2^-f.  FP64 p has
    // relative error <= 1e-13 (tested against mpmath), so p64(c*) <= p64(c_b)
    // gives ln p_true(c*) <= B 2^-f + 3e-13.  Its stage-1 bound satisfies
    // LB(c*) <= ln pmf(kk) 2^f + 4.5 <= B + 5 < B(t) + 6 = tau at every row,
    // so c* entered stage 2, and lo(c*) <= ln p_true(c*) 2^f <= B + 1 <=
    // B(t) + 1 at its evaluation and at every later compaction, so it stayed.
    // B is clamped to >= -700 nats so that cells whose FP64 p underflows (and
    // so ties at 0) are kept too.
    bool done = false;
    int guess = kNoGuess;
    if (A.guess_hist != nullptr && !coop) {
      int gq = bound_guess_bin(A.guess_hist, lane);
      if (gq >= 0) guess = max((int)floor(-0.25 * (double)gq * scale), Bfloor);
    }
    if (guess != kNoGuess) {
      // speculative single sweep from the guessed bound
      B = guess;
      candidate_sweep();
      done = B_valid;  // some cell reached the guess: B is a valid bound
      if (!done) {
        nsurv = 0;
        ++nfall;
      }
    }
    if (!done) {
      // pass A: each lane's cell with the smallest LB, whose stage-2 upper
      // bound seeds B
      int bestLB = 0x7fffffff, bestCell = -1, bestK = 0;
      sweep<C>(x, sRow, n1, cnt, lane, A.hwlab != 0, [&](int i, const int (&O)[C], int excl) {
        if (!my_row(i)) return;
        const int K = sRow[i + 1];
        const int NK = N - K;
        const uint32_t Arow = F[K] + F[NK] - FN;
        const float Kf = (float)K;
#pragma unroll
        for (int t = 0; t < C; ++t) {
          int k = O[t] + excl;
          int lb = lb_fix(F, K, NK, Arow, Kf, ncol[t], Bc[t], qc[t], k);
          if (t < tvalid && lb < bestLB) {
            bestLB = lb;
            bestCell = (i << 16) | (lane * C + t);
            bestK = k;
          }
        }
      });
      B = kScreenSlack;
      if (bestCell >= 0) {
        int ci = bestCell >> 16, cj = bestCell & 0xffff;
        Interval iv = eval32(F, N, FN, sRow[ci + 1], __ldg(A.P.ncnt + cj), bestK, scale);
        B = iv.hi;
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) B = min(B, __shfl_xor_sync(kFull, B, d));
      B = max(B, Bfloor);
      if (coop) {
        if (lane == 0) atomicMin(&sB, B);
        __syncthreads();
        B = sB;
      }
      B_valid = true;
      candidate_sweep();
    }
    if (coop) {
      __syncthreads();  // every warp's stage 2 is done: sB is the task's bound
      B = min(B, sB);
    }
    refine_survivors();
    if (coop) {
      if (lane == 0) {
        sBestP[warp] = best64.p;
        sBestK[warp] = best64.k;
        sBestI[warp] = best64.i;
        sBestJ[warp] = best64.j;
      }
      __syncthreads();
      if (warp == 0) {
        Best bb = best_init();
        if (lane < kGridWarps) bb = Best{sBestP[lane], sBestK[lane], sBestI[lane], sBestJ[lane]};
        warp_best(bb);
        if (lane == 0) A.out[b] = TaskResult{bb.p, bb.i, bb.j, bb.k, A.route};
      }
      continue;
    }
    if (A.guess_hist != nullptr && lane == 0) bound_record(A.guess_hist, B, scale);
    if (lane == 0) A.out[b] = TaskResult{best64.p, best64.i, best64.j, best64.k, A.route};
  }
  if (lane == 0 && A.n_refined) {
    atomicAdd(A.n_refined, n64);
    atomicAdd(A.n_refined + 1, n32);
    atomicAdd(A.n_refined + 2, nfall);
  }
}

template <int C>
cudaError_t launch_grid_impl(const GridArgs& a, int ctas, size_t smem, cudaStream_t s) {
  cudaError_t e = raise_smem_limit((const void*)grid_kernel<C>, smem);
  if (e != cudaSuccess) return e;
  grid_kernel<C><<<ctas, kGridWarps * 32, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace dto

#define DTO_DEFINE_GRID(CC)                                                                        \
  namespace dto {                                                                                  \
  cudaError_t launch_grid_c##CC(const GridArgs& a, int ctas, size_t smem, cudaStream_t s) {        \
    return launch_grid_impl<CC>(a, ctas, smem, s);                                                 \
  }                                                                                                \
  }
