// dto_table.cuh -- the table screen: the fast path of the threshold-pair search.
//
// For a pair and a bound guess tau (fixed-point ln p), kthr[i][j] is the
// smallest overlap k of cell (i, j) whose lower bound LBT(k) of ln P(X >= k)
// is <= tau + margin, where
//   LBT(k) = ln P_w(max(k, mode)),  P_w(k) = sum_{j=k}^{k+w-1} pmf(j)  (w = 48),
// evaluated in FP32 with its rounding error subtracted.  Above the mode P_w is
// decreasing in k (the window loses pmf(k) and gains the smaller pmf(k+w)),
// and P(X >= k) >= P_w(max(k, mode)) for every k, so every cell with
// k < kthr has ln p > tau (the margin of 0.002 nats covers the FP32 error,
// <= 1.1e-4 nats).  A task then needs, per cell, one shared-memory counter
// load, two adds and one compare against the table row held in registers.
//
// A task is accepted when some cell's stage-2 upper bound reaches tau: the
// FP64 argmin then lies among the hits (cells with k >= kthr).  Each hit is
// rechecked with the fixed-point log-pmf bound against the task's running B
// and goes through stage 2 (FP32 tail interval) and stage 3 (FP64) exactly as
// in the exhaustive screen (dto_grid.cuh).  A task whose minimum lies above
// tau is appended to a fallback list that the exhaustive screen processes.
#pragma once
#include "dto_grid.cuh"

namespace dto {

constexpr double kTableMargin = 0.002;  // nats added to tau when the table is built

__host__ __device__ constexpr int table_cq(int C) { return (C + 7) & ~7; }

// The first overlap k of cell (i, j) whose LBT(k) is <= tauT (binary search
// over k), 0 when every k passes, min(K, n) + 1 when none does.
__device__ __forceinline__ int table_thr(const TableArgs& A, uint32_t FN, double scale, int tauT, int i, int j) {
  const int K = __ldg(A.rowstart + i + 1);
  const int n = __ldg(A.ncnt + j);
  const int a = min(K, n), b = max(K, n);
  const long long mode = ((long long)(a + 1) * (long long)(b + 1)) / (long long)(A.N + 2);
  if (lbt_fix(A.F, A.N, FN, K, n, (int)mode, mode, scale) <= tauT) return 0;
  // invariant: pred(lo) false, pred(hi) true or hi = a + 1
  int lo = (int)mode, hi = a + 1;
  while (hi - lo > 1) {
    const int mid = lo + (hi - lo) / 2;
    if (lbt_fix(A.F, A.N, FN, K, n, mid, mode, scale) <= tauT) hi = mid;
    else lo = mid;
  }
  return hi;
}

// Layout [i][q][lane][8] for 16 lanes of A.C (= 2 C) columns each: entry t
// of a lane's row is in its q = t / 8-th 16-byte chunk, so a load of chunk q
// by the lanes reads 16 x 16 contiguous bytes.
//
// Entries come in pairs, the two 16-bit halves of one word of the sweep
// (columns t, t + 1, t even; one thread a pair).  The sweep holds a
// cell's overlap o in a 16-bit half (o <= N1 <= 65534) and adds the entry
// with one 32-bit add to both halves at once; bit 15 (31) of the sum must
// be set exactly when o >= kthr.  A cell's overlap lies in
// [L, U] = [max(0, K_i + m_j - N1), min(K_i, m_j)] whatever the permutation
// (m_j: the list-1 positions whose label is <= j), and U - L <= N1 / 2 <=
// 32767.  With kthr clamped to [L, U + 1] (which changes no hit),
// o - kthr lies in [-32768, 32767], so the half's sum 0x8000 + o - kthr
// lies in [0, 0xFFFF] and its bit 15 is the test.  The entry is
// 0x8000 - kthr modulo 2^16: when kthr > 0x8000 that wraps, and the lower
// half's sum then always carries one into the upper half, which the upper
// entry takes back (it is one less).  A column past the grid (padding) has
// the overlap of the last column and the entry "never" (kthr = U + 1).
static __global__ void table_build_kernel(const TableArgs A) {
  constexpr int lanes = 16;
  const int Cq = table_cq(A.C);
  const long long cells = (long long)A.n1 * lanes * Cq;
  const double scale = ldexp(1.0, A.fshift);
  const int tauT = A.tau + (int)ceil(kTableMargin * scale);
  const uint32_t FN = __ldg(A.F + A.N);
  for (long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 2; c < cells;
       c += (long long)gridDim.x * blockDim.x * 2) {
    const int i = (int)(c / (lanes * Cq));
    const int rem = (int)(c % (lanes * Cq));
    const int q = rem / (8 * lanes), lane = (rem / 8) % lanes;
    const int t = 8 * q + rem % 8;
    const int j = lane * A.C + t;
    const int K = __ldg(A.rowstart + i + 1);
    int k2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int jj = j + h;
      const int m = __ldg(A.mcnt + min(jj, A.n2 - 1));
      const int U = min(K, m), L = max(0, K + m - A.N1);
      const int thr = (t + h < A.C && jj < A.n2) ? table_thr(A, FN, scale, tauT, i, jj) : 0x10000;
      k2[h] = min(max(thr, L), U + 1);
    }
    A.kthr[c] = (uint16_t)((0x8000 - k2[0]) & 0xFFFF);
    A.kthr[c + 1] = (uint16_t)((0x8000 - k2[1] - (k2[0] > 0x8000 ? 1 : 0)) & 0xFFFF);
  }
}

constexpr int kTableSurvCap = 64;
// Hits after which a sweep resolves early to switch to a tighter table
// (768 measured within noise of it, 384 1-3 % slower).
constexpr int kEarlyHits = 512;
constexpr int kPend = 64;  // deferred FP64 evaluations per warp (several tasks)

// Per-task state in shared memory: the hot sweep never touches it; only the
// hit path and the task end do.  n32, n64 and npend count for the whole warp
// and live in the warp's first WarpTask (TableWarpMem::q).
struct WarpTask {
  int B;        // running bound (fixed-point ln p)
  int B_valid;  // some cell's stage-2 upper bound reached B
  int ncand, nsurv;
  double bp;    // FP64 best so far
  int bk, bi, bj;
  int nhits;    // hits appended by the sweep
  unsigned long long n32, n64;
  int npend;    // entries in the deferred FP64 queue
  int pad2;
};

// A task's view of its warp's shared memory (hw_warp_mem): its column
// counters, its WarpTask and survivors, and the warp's candidate and
// deferred-FP64 buffers.
struct TableWarpMem {
  int* cnt;
  int2* cand;
  int* survCell;
  int* survK;
  int* survLo;
  WarpTask* st;   // this task
  WarpTask* q;    // the warp's counters (n32, n64, npend)
  double* pendP;  // deferred FP64 queue: p, task, packed cell, overlap
  int* pendTask;
  int* pendCell;
  int* pendK;
};

// Pair tables one CTA reads in the resolve paths: row sizes K (rowstart),
// column sizes n and the fixed-point ln m! table, in shared memory when the
// table fits (generic pointers: shared or global).
struct TabGrid {
  const int* row;
  const int* ncnt;
  const uint32_t* F;
};

// The resolve helpers below are inlined into the sweeps: as calls they made
// the kernel copy its arguments and per-task pointers to local memory and
// save live registers around every call (spills in the row loop).

// Stage 3 on the survivors the current B admits.
static __device__ __forceinline__ void table_refine(const TableGridArgs& A, const TabGrid& g, const TableWarpMem& m,
                                          int lane) {
  __syncwarp();
  WarpTask st = *m.st;
  Best lb{st.bp, st.bk, st.bi, st.bj};
  int done = 0;
  for (int q = lane; q < st.nsurv; q += 32) {
    if (m.survLo[q] <= st.B + 1) {
      int ci = m.survCell[q] >> 16, cj = m.survCell[q] & 0xffff;
      double p = sf64(A.P.LF, A.P.Npop, g.row[ci + 1], g.ncnt[cj], m.survK[q]);
      best_take(lb, p, m.survK[q], ci, cj);
      ++done;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) done += __shfl_xor_sync(kFull, done, d);
  warp_best(lb);
  __syncwarp();
  if (lane == 0) {
    m.st->bp = lb.p;
    m.st->bk = lb.k;
    m.st->bi = lb.i;
    m.st->bj = lb.j;
    m.st->nsurv = 0;
    m.q->n64 += (unsigned long long)done;
  }
  __syncwarp();
}

// The deferred FP64 queue: one tail per lane, then the first entry of each
// task's run (a task's entries are contiguous) takes the task's argmin with
// the reference's tie-break and writes its result.  Tasks share the FP64
// instructions this way: on GB300 an FP64 warp instruction costs the same
// whether one lane or all 32 are active.
static __device__ __forceinline__ void table_pending_flush(const TableGridArgs& A, const TabGrid& g,
                                                        const TableWarpMem& m, int lane) {
  __syncwarp();
  const int np = m.q->npend;
  for (int q = lane; q < np; q += 32) {
    const int ci = m.pendCell[q] >> 16, cj = m.pendCell[q] & 0xffff;
    m.pendP[q] = sf64(A.P.LF, A.P.Npop, g.row[ci + 1], g.ncnt[cj], m.pendK[q]);
  }
  __syncwarp();
  for (int q = lane; q < np; q += 32) {
    const int tw = m.pendTask[q];  // task | route << 28
    if (q == 0 || m.pendTask[q - 1] != tw) {
      Best b = best_init();
      for (int r = q; r < np && m.pendTask[r] == tw; ++r)
        best_take(b, m.pendP[r], m.pendK[r], m.pendCell[r] >> 16, m.pendCell[r] & 0xffff);
      A.out[tw & 0x0FFFFFFF] = TaskResult{b.p, b.i, b.j, b.k, (int)((unsigned)tw >> 28)};
    }
  }
  __syncwarp();
  if (lane == 0) {
    m.q->n64 += (unsigned long long)np;
    m.q->npend = 0;
  }
  __syncwarp();
}

// Queue the task's survivors that the final B admits, without duplicates
// (a cell can reach stage 2 twice: as a seed and as a hit).
static __device__ __forceinline__ void table_defer(const TableGridArgs& A, const TabGrid& g, const TableWarpMem& m,
                                                int lane, int task, int route) {
  __syncwarp();
  const int B = m.st->B;
  const int ns = m.st->nsurv;
  if (m.q->npend + ns > kPend) table_pending_flush(A, g, m, lane);
  int npend = m.q->npend;
  for (int q0 = 0; q0 < ns; q0 += 32) {
    const int q = q0 + lane;
    bool keep = q < ns && m.survLo[q] <= B + 1;
    if (keep) {
      const int cell = m.survCell[q];
      for (int r = 0; r < q; ++r)
        if (m.survCell[r] == cell && m.survLo[r] <= B + 1) {
          keep = false;
          break;
        }
    }
    const unsigned msk = __ballot_sync(kFull, keep);
    if (keep) {
      const int pos = npend + __popc(msk & ((1u << lane) - 1u));
      m.pendTask[pos] = task | (route << 28);  // task ids stay below 2^28
      m.pendCell[pos] = m.survCell[q];
      m.pendK[pos] = m.survK[q];
    }
    npend += __popc(msk);
  }
  __syncwarp();
  if (lane == 0) {
    m.q->npend = npend;
    m.st->nsurv = 0;
  }
  __syncwarp();
}

// Stage 2 on the candidate buffer.
static __device__ __forceinline__ void table_flush(const TableGridArgs& A, const TabGrid& g, const TableWarpMem& m,
                                         int lane) {
  __syncwarp();
  const int N = (int)A.P.Npop;
  const uint32_t* F = g.F;
  const uint32_t FN = F[N];
  const double scale = ldexp(1.0, A.P.fshift);
  const int Bfloor = (int)floor(-700.0 * scale);
  const int ncand = m.st->ncand;
  int B = m.st->B;
  int B_valid = m.st->B_valid;
  for (int q0 = 0; q0 < ncand; q0 += 32) {
    int q = q0 + lane;
    Interval iv{0x7fffffff, 0x7fffffff};
    int2 c = make_int2(0, 0);
    if (q < ncand) {
      c = m.cand[q];
      int ci = c.x >> 16, cj = c.x & 0xffff;
      iv = eval32_filtered(F, N, FN, g.row[ci + 1], g.ncnt[cj], c.y, scale, B);
    }
    int h = iv.hi;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) h = min(h, __shfl_xor_sync(kFull, h, d));
    if (h <= B) {
      B = max(h, Bfloor);
      B_valid = 1;
    }
    bool keep = (q < ncand) && iv.lo <= B + 1;
    unsigned msk = __ballot_sync(kFull, keep);
    int nk = __popc(msk);
    int nsurv = m.st->nsurv;
    if (nsurv + nk > kTableSurvCap) {
      __syncwarp();
      if (lane == 0) m.st->B = B;
      table_refine(A, g, m, lane);
      nsurv = 0;
    }
    if (keep) {
      int pos = nsurv + __popc(msk & ((1u << lane) - 1u));
      m.survCell[pos] = c.x;
      m.survK[pos] = c.y;
      m.survLo[pos] = iv.lo;
    }
    __syncwarp();
    if (lane == 0) m.st->nsurv = nsurv + nk;
    __syncwarp();
  }
  __syncwarp();
  if (lane == 0) {
    m.st->B = B;
    m.st->B_valid = B_valid;
    m.st->ncand = 0;
    m.q->n32 += (unsigned long long)ncand;
  }
  __syncwarp();
}

// Fixed-point lower bound of ln p for one cell from its counts alone.
__device__ __forceinline__ int cell_lb(const uint32_t* F, int N, uint32_t FN, int K, int n, int k) {
  const uint32_t Arow = F[K] + F[N - K] - FN;
  const uint32_t Bcol = F[n] + F[N - n];
  return lb_fix(F, K, N - K, Arow, (float)K, n, Bcol, (float)n * (1.0f / (float)N), k);
}

// Resolve a task from its hits (cells with k >= kthr), held in global memory.
// The lowest stage-1 bound of each lane's hits seeds B through stage 2; then
// every hit whose stage-1 bound is within B goes through stage 2 (behind the
// partial-sum filter) in batches, B tightening as it goes.  The claim of
// dto_grid.cuh applies unchanged: the FP64 argmin is among the hits and is
// never filtered out.
static __device__ __forceinline__ void table_resolve(const TableGridArgs& A, const TabGrid& g,
                                                  const TableWarpMem& m, int lane, const int2* hb, int nh) {
  const int N = (int)A.P.Npop;
  const uint32_t* F = g.F;
  const uint32_t FN = F[N];
  // seed: each lane's lowest-bound hit
  int bestLB = 0x7fffffff;
  int2 best = make_int2(0, 0);
  for (int q = lane; q < nh; q += 32) {
    const int2 h = hb[q];
    const int lb = cell_lb(F, N, FN, g.row[(h.x >> 16) + 1], g.ncnt[h.x & 0xffff], h.y);
    if (lb < bestLB) {
      bestLB = lb;
      best = h;
    }
  }
  {
    const bool have = bestLB != 0x7fffffff;
    const unsigned msk = __ballot_sync(kFull, have);
    __syncwarp();
    if (have) m.cand[__popc(msk & ((1u << lane) - 1u))] = best;
    __syncwarp();
    if (lane == 0) m.st->ncand = __popc(msk);
    __syncwarp();
    table_flush(A, g, m, lane);
  }
  // every hit within the bound
  for (int q0 = 0; q0 < nh; q0 += 32) {
    const int q = q0 + lane;
    int2 h = make_int2(0, 0);
    bool keep = false;
    if (q < nh) {
      h = hb[q];
      keep = cell_lb(F, N, FN, g.row[(h.x >> 16) + 1], g.ncnt[h.x & 0xffff], h.y) <=
             m.st->B + kScreenSlack + 1;
    }
    const unsigned msk = __ballot_sync(kFull, keep);
    if (msk) {
      const int base = m.st->ncand;
      __syncwarp();
      if (keep) m.cand[base + __popc(msk & ((1u << lane) - 1u))] = h;
      __syncwarp();
      if (lane == 0) m.st->ncand = base + __popc(msk);
      __syncwarp();
      if (m.st->ncand > kCandCap - 32) table_flush(A, g, m, lane);
    }
  }
  if (m.st->ncand > 0) table_flush(A, g, m, lane);
}

// The tighter tables of the arguments, by selects (a dynamic index into the
// kernel's argument arrays would copy the arguments to local memory).
__device__ __forceinline__ const uint16_t* tight_of(const TableGridArgs& A, int q) {
  return q == 0 ? A.tight[0] : q == 1 ? A.tight[1] : A.tight[2];
}
__device__ __forceinline__ int tight_tau_of(const TableGridArgs& A, int q) {
  return q == 0 ? A.tight_tau[0] : q == 1 ? A.tight_tau[1] : A.tight_tau[2];
}
// The same per cascade level l (0: the fields above; 1, 2: the *_up fields).
__device__ __forceinline__ const uint16_t* lv_kthr(const TableGridArgs& A, int l) {
  return l == 0 ? A.kthr : l == 1 ? A.kthr_up[0] : A.kthr_up[1];
}
__device__ __forceinline__ int lv_tau(const TableGridArgs& A, int l) {
  return l == 0 ? A.tau : l == 1 ? A.tau_up[0] : A.tau_up[1];
}
__device__ __forceinline__ int lv_ntight(const TableGridArgs& A, int l) {
  return l == 0 ? A.ntight : l == 1 ? A.ntight_up[0] : A.ntight_up[1];
}
__device__ __forceinline__ const uint16_t* lv_tight(const TableGridArgs& A, int l, int q) {
  if (l == 0) return tight_of(A, q);
  if (l == 1) return q == 0 ? A.tight_up[0][0] : q == 1 ? A.tight_up[0][1] : A.tight_up[0][2];
  return q == 0 ? A.tight_up[1][0] : q == 1 ? A.tight_up[1][1] : A.tight_up[1][2];
}
__device__ __forceinline__ int lv_tight_tau(const TableGridArgs& A, int l, int q) {
  if (l == 0) return tight_tau_of(A, q);
  if (l == 1) return q == 0 ? A.tight_tau_up[0][0] : q == 1 ? A.tight_tau_up[0][1] : A.tight_tau_up[0][2];
  return q == 0 ? A.tight_tau_up[1][0] : q == 1 ? A.tight_tau_up[1][1] : A.tight_tau_up[1][2];
}

// ---------------------------------------------------------------------------
// The packed sweep with a half-warp per task.
//
// Lane h (0..15) of half-warp t owns the C2 consecutive columns
// [h C2, (h + 1) C2) of task t as C2 / 2 words of two 16-bit counts, so two
// tasks share every instruction of the row loop: the row bounds, the loop
// control, the table-row loads (both halves read the same 256 bytes) and the
// scan.  Per row:
//   1. each label of the row adds 1 to its column's half-word (one shared
//      atomic; a table run's labels are the counts' byte offsets, bit 13
//      the upper half: hw_label_of_column);
//   2. each lane runs the in-lane prefix of its counts in NG independent
//      chains (x 0x10001 + R, then the upper half carried), keeping every
//      word's two partial overlaps in registers; the chains' totals give the
//      lane's total, and a 4-step scan over the half-warp its offset E;
//   3. overlap + (0x8000 - kthr) sets bit 15 (31) of a half exactly when the
//      overlap reaches the table's threshold (the entries' form, built by
//      table_build_kernel, keeps every sum inside its half), tested for all
//      words with one OR; only a lane with a set bit records its hits,
//      straight from the registers.
// Overlaps are at most N1 <= 65534, so the counters and partial sums never
// carry from one half into the other.  The hits are resolved one task at a
// time by the whole warp.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int hw_task_ints(int C2) {
  return 16 * hw_wp(C2) + (int)(sizeof(WarpTask) / 4) + 3 * kTableSurvCap;
}
__host__ __device__ constexpr int hw_warp_ints(int C2) { return 2 * hw_task_ints(C2) + 2 * kCandCap + 5 * kPend; }

__device__ __forceinline__ TableWarpMem hw_warp_mem(int* base, int C2, int t) {
  TableWarpMem m;
  int* tb = base + t * hw_task_ints(C2);
  m.cnt = tb;
  m.st = reinterpret_cast<WarpTask*>(tb + 16 * hw_wp(C2));
  m.q = reinterpret_cast<WarpTask*>(base + 16 * hw_wp(C2));
  m.survCell = reinterpret_cast<int*>(m.st + 1);
  m.survK = m.survCell + kTableSurvCap;
  m.survLo = m.survK + kTableSurvCap;
  int* sh = base + 2 * hw_task_ints(C2);
  m.cand = reinterpret_cast<int2*>(sh);
  m.pendP = reinterpret_cast<double*>(m.cand + kCandCap);
  m.pendTask = reinterpret_cast<int*>(m.pendP + kPend);
  m.pendCell = m.pendTask + kPend;
  m.pendK = m.pendCell + kPend;
  return m;
}

// Multi: the launch sweeps the tasks of several pairs (segments; Ain.segs
// holds one TableGridArgs per pair, all of the same C).  A warp works through
// the segments in order, both its half-warps on tasks of one segment, with
// that segment's arguments copied to shared memory; the pairs' tables (row
// bounds, set sizes, ln m!) are read from global memory.  A segment's tail
// is filled by the warps that have moved on to the next.
template <int C2, bool Multi>
__global__ void __launch_bounds__(kTableWarps * 32, 1) table_hw_kernel(const TableGridArgs Ain) {
  constexpr int NQ = hw_cq(C2) / 8;  // 16-byte table chunks per lane per row
  constexpr int NW = C2 / 2;         // counter words per lane
  constexpr int Wp = hw_wp(C2);
  constexpr int TI = hw_task_ints(C2);
  constexpr int NG = (NW % 4 == 0) ? 4 : (NW % 2 == 0 ? 2 : 1);  // independent chains
  constexpr int GW = NW / NG;
  static_assert(C2 % 2 == 0 && NW <= 4 * NQ, "packed columns come in pairs");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int h = lane & 15, half = lane >> 4;
  __shared__ TableGridArgs sSeg[Multi ? kTableWarps : 1];  // the warp's segment (Multi)
  const TableGridArgs& A = Multi ? sSeg[warp] : Ain;
  // one pair: its row bounds, set sizes and (where it fits) ln m! table in
  // shared memory; Multi: none (each pair's are read from global memory)
  const int Npop0 = (int)Ain.P.Npop;
  uint32_t* sF = reinterpret_cast<uint32_t*>(smem_raw);
  int* sRow = reinterpret_cast<int*>(sF + ((!Multi && Ain.smemF) ? ((Npop0 + 1 + 3) & ~3) : 0));
  int* sNcnt = sRow + (Multi ? 0 : ((Ain.P.n1 + 1 + 3) & ~3));
  int* sWarp = sNcnt + (Multi ? 0 : ((Ain.P.n2 + 3) & ~3));
  int* const wb = sWarp + warp * hw_warp_ints(C2);
  if constexpr (!Multi) {
    for (int q = threadIdx.x; q <= Ain.P.n1; q += blockDim.x) sRow[q] = __ldg(Ain.P.rowstart + q);
    for (int q = threadIdx.x; q < Ain.P.n2; q += blockDim.x) sNcnt[q] = __ldg(Ain.P.ncnt + q);
    if (Ain.smemF)
      for (int q = threadIdx.x; q <= Npop0; q += blockDim.x) sF[q] = __ldg(Ain.P.F + q);
  }
  // the cascade levels' tables and bounds, per warp, indexed by level from
  // shared memory (selecting among the kernel's arguments at run time kept
  // them all in registers and slowed the row loop by a fifth)
  // (one copy per CTA for one pair, per warp for several)
  constexpr int kLv = Multi ? kTableWarps : 1;
  __shared__ const uint16_t* sLvTabW[kLv][3][4];  // [level][0: the level's table, 1..3: its tighter tables]
  __shared__ int sLvTauW[kLv][3][4];              // [level][0: its bound, 1..3: the tighter tables' bounds]
  __shared__ int sLvNtightW[kLv][3];
  const uint16_t* (*const sLvTab)[4] = sLvTabW[Multi ? warp : 0];
  int (*const sLvTau)[4] = sLvTauW[Multi ? warp : 0];
  int* const sLvNtight = sLvNtightW[Multi ? warp : 0];
  // the segment-dependent state: the pair's grid rows, its tables, the task count
  int n1 = 0, ntask = 0;
  const int* rowp = sRow;
  TabGrid g{sRow, sNcnt, Ain.smemF ? sF : Ain.P.F};
  auto bind_seg = [&]() {
    if (lane < 3 && (Multi || warp == 0)) {  // one pair: read after the barrier below
      const int l = lane;
      sLvTab[l][0] = lv_kthr(A, l);
      sLvTau[l][0] = lv_tau(A, l);
      sLvNtight[l] = lv_ntight(A, l);
      for (int q = 0; q < 3; ++q) {
        sLvTab[l][1 + q] = lv_tight(A, l, q);
        sLvTau[l][1 + q] = lv_tight_tau(A, l, q);
      }
    }
    n1 = A.P.n1;
    ntask = A.ntask_dev ? *((volatile const int*)A.ntask_dev) : A.ntask;
    if constexpr (Multi) {
      rowp = A.P.rowstart;
      g = TabGrid{A.P.rowstart, A.P.ncnt, A.P.F};
    }
    __syncwarp();
  };
  int seg = 0;
  auto load_seg = [&](int sgi) {  // Multi: copy segment sgi's arguments
    __syncwarp();
    const int* src = reinterpret_cast<const int*>(Ain.segs + sgi);
    int* dst = reinterpret_cast<int*>(&sSeg[Multi ? warp : 0]);
    for (int q = lane; q < (int)(sizeof(TableGridArgs) / 4); q += 32) dst[q] = __ldg(src + q);
    __syncwarp();
  };
  if constexpr (Multi) load_seg(0);
  bind_seg();
  int* const cnt_t = wb + half * TI;  // this lane's task's counters
  WarpTask* const st_me = reinterpret_cast<WarpTask*>(cnt_t + 16 * Wp);
  auto st_of = [&](int t) { return reinterpret_cast<WarpTask*>(wb + t * TI + 16 * Wp); };
  if (lane == 0) {
    st_of(0)->n32 = 0;
    st_of(0)->n64 = 0;
    st_of(0)->npend = 0;
  }
  __syncthreads();
  const int hcap = Ain.hitcap / 2;  // per task
  int2* const hbw = Ain.hitbuf + (size_t)(blockIdx.x * kTableWarps + warp) * Ain.hitcap;
  int2* const hb_me = hbw + half * hcap;
  unsigned long long nfall = 0;
  // Each half-warp holds one task and its cascade level (warp-uniform
  // copies in every lane); a free half takes the next level-0 task, a task
  // with no hit at level l is swept again at level l + 1 by the same half.
  int tb[2] = {-1, -1}, tl[2] = {0, 0};
  bool drained = false;
  for (;;) {
    const int want = (tb[0] < 0 ? 1 : 0) + (tb[1] < 0 ? 1 : 0);
    if (want && !drained) {
      int b = 0;
      if (lane == 0) b = atomicAdd(A.work, want);
      b = __shfl_sync(kFull, b, 0);
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        if (tb[t] < 0) {
          if (b < ntask) {
            tb[t] = A.task_list ? A.task_list[b] : b;
            tl[t] = 0;
          } else {
            drained = true;
          }
          ++b;
        }
      }
    }
    if (tb[0] < 0 && tb[1] < 0) {
      if constexpr (Multi) {
        if (seg + 1 < Ain.nseg) {
          // the deferred FP64 evaluations belong to this segment's tasks
          if (st_of(0)->npend > 0) table_pending_flush(A, g, hw_warp_mem(wb, C2, 0), lane);
          __syncwarp();
          // and so do the refine and fall-through counts so far
          if (lane == 0 && A.n_refined) {
            atomicAdd(A.n_refined, st_of(0)->n64);
            atomicAdd(A.n_refined + 1, st_of(0)->n32);
            atomicAdd(A.n_refined + 2, nfall);
            st_of(0)->n64 = 0;
            st_of(0)->n32 = 0;
          }
          nfall = 0;
          load_seg(++seg);
          bind_seg();
          drained = false;
          continue;
        }
      }
      break;
    }
    const int bt_me = half ? tb[1] : tb[0];
    const int lv_me = half ? tl[1] : tl[0];
    const bool live = bt_me >= 0;
    const int* const x32 = reinterpret_cast<const int*>(A.X + (long long)(live ? bt_me : 0) * A.xstride);
    if (h == 0) {
      st_me->B = sLvTau[lv_me][0];
      st_me->B_valid = 0;
      st_me->ncand = 0;
      st_me->nsurv = 0;
      st_me->nhits = 0;
      const Best z = best_init();
      st_me->bp = z.p;
      st_me->bk = z.k;
      st_me->bi = z.i;
      st_me->bj = z.j;
    }
    for (int q = h; q < 16 * Wp; q += 16) cnt_t[q] = 0;
    __syncwarp();
    // labels as 32-bit words (two each), a row's words prefetched one row
    // ahead: 16 words (32 labels) per task, and 16 more for rows that long
    int s = rowp[0], e = rowp[1];
    int w0, w1;
    {
      const int q0 = (s >> 1) + h;
      w0 = (live && 2 * q0 < e) ? __ldg(x32 + q0) : -1;
      w1 = (live && 2 * (q0 + 16) < e) ? __ldg(x32 + q0 + 16) : -1;
    }
    bool anyhits[2] = {false, false};
    int cur_tight[2] = {-1, -1};  // the table each task's rows are compared with (uniform)
    const uint4* ktab_me = reinterpret_cast<const uint4*>(sLvTab[lv_me][0]);
    // a label (the sweep's form) is its count's byte offset, bit 13 the
    // upper half of the word
    auto add_lab = [&](int v) {
      atomicAdd(reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(cnt_t) + (v & 0x1FFF)),
                1u << ((v >> 9) & 16));
    };
    auto add_word = [&](int w, int q, int rs, int re) {
      const int p = 2 * q;
      const int lab0 = (int)(short)(w & 0xffff), lab1 = w >> 16;  // sign-extended labels
      if (p >= rs && p < re && lab0 >= 0) add_lab(lab0);
      if (p + 1 >= rs && p + 1 < re && lab1 >= 0) add_lab(lab1);
    };
    // A half without a task (its slot drained) sweeps no labels: its zero
    // overlaps lie outside the cells' ranges the table entries assume, so its
    // "hits" are meaningless and are not recorded.
    auto push_hit = [&](int i, int col, int k) {
      if (!live) return;
      const int pos = atomicAdd(&st_me->nhits, 1);
      if (pos < hcap) hb_me[pos] = make_int2((i << 16) | (h * C2 + col), k);
    };
    // The row loop breaks out every fourth row when a task needs an early
    // resolve, resolves after it and resumes at the next row: the resolve
    // code stays out of the loop's body.
    int i = 0;
    for (;;) {
    bool resolve_now = false;
    for (; i < n1; ++i) {
      const int c0 = w0, c1 = w1;
      const int sN = e;
      const int eN = (i + 2 <= n1) ? rowp[i + 2] : e;
      {
        const int q0 = (sN >> 1) + h;
        w0 = (live && 2 * q0 < eN) ? __ldg(x32 + q0) : -1;
        w1 = -1;
        if (eN > 2 * (sN >> 1) + 32 && live && 2 * (q0 + 16) < eN) w1 = __ldg(x32 + q0 + 16);
      }
      // this row's table chunks, consumed after the labels and the chains
      uint4 kt[NQ];
#pragma unroll
      for (int u = 0; u < NQ; ++u) kt[u] = __ldg(ktab_me + ((size_t)i * NQ + u) * 16 + h);
      {
        const int q0 = (s >> 1) + h;
        add_word(c0, q0, s, e);
        if (e > 2 * (s >> 1) + 32) {  // a row of more than 32 labels (uniform)
          add_word(c1, q0 + 16, s, e);
          if (live)
            for (int q = q0 + 32; 2 * q < e; q += 16) add_word(__ldg(x32 + q), q, s, e);
        }
      }
      __syncwarp();
      // in-lane partial overlaps: NG chains of GW words, each from zero
      uint32_t v[NW];
      uint32_t Rg[NG];
#pragma unroll
      for (int gq = 0; gq < NG; ++gq) Rg[gq] = 0;
#pragma unroll
      for (int u = 0; u < NQ; ++u) {
        const uint4 c4 = *reinterpret_cast<const uint4*>(cnt_t + h * Wp + 4 * u);
        const uint32_t cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int w = 4 * u + c;
          if (w < NW) {
            const int gq = w / GW;
            v[w] = cv[c] * 0x10001u + Rg[gq];
            Rg[gq] = __byte_perm(v[w], 0, 0x3232);
          }
        }
      }
      // offsets of the chains (both halves), the lane's total, the scan
      uint32_t off[NG];
      off[0] = 0;
#pragma unroll
      for (int gq = 1; gq < NG; ++gq) off[gq] = off[gq - 1] + Rg[gq - 1];
      const int mine = (int)((off[NG - 1] + Rg[NG - 1]) & 0xFFFFu);
      int incl = mine;
#pragma unroll
      for (int d = 1; d < 16; d <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, d, 16);
        if (h >= d) incl += y;
      }
      const uint32_t E = (uint32_t)(incl - mine) * 0x10001u;
      uint32_t Eg[NG];
#pragma unroll
      for (int gq = 0; gq < NG; ++gq) Eg[gq] = E + off[gq];
      uint32_t acc = 0;
#pragma unroll
      for (int u = 0; u < NQ; ++u) {
        const uint32_t tv[4] = {kt[u].x, kt[u].y, kt[u].z, kt[u].w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int w = 4 * u + c;
          if (w < NW) acc |= v[w] + Eg[w / GW] + tv[c];
        }
      }
      if (acc & 0x80008000u) {
#pragma unroll
        for (int u = 0; u < NQ; ++u) {
          const uint32_t tv[4] = {kt[u].x, kt[u].y, kt[u].z, kt[u].w};
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int w = 4 * u + c;
            if (w < NW) {
              const uint32_t o = v[w] + Eg[w / GW];
              const uint32_t d = o + tv[c];
              if (d & 0x80008000u) {  // one test a word; the halves only for words with a hit
                if (d & 0x8000u) push_hit(i, 2 * w, (int)(o & 0xFFFFu));
                if (d & 0x80000000u) push_hit(i, 2 * w + 1, (int)(o >> 16));
              }
            }
          }
        }
      }
      // the next row's counter updates wait for every lane's reads of this row
      __syncwarp();
      s = sN;
      e = eN;
      // every fourth row: could a task's buffer overflow within the next four
      // rows, or has it gathered kEarlyHits hits while a tighter table is
      // left?  Then resolve what it holds (below); the bound B it sets lets
      // its remaining rows be compared with the tightest table whose bound
      // is still >= B (every cell with ln p <= B stays a hit).
      if ((i & 3) == 3) {
        bool need = false;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const int nh = st_of(t)->nhits;
          need = need || nh > hcap - 4 * 16 * C2 || (cur_tight[t] + 1 < sLvNtight[tl[t]] && nh >= kEarlyHits);
        }
        if (need) {
          ++i;
          resolve_now = true;
          break;
        }
      }
    }
    if (!resolve_now) break;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int nh = st_of(t)->nhits;
      if (nh > hcap - 4 * 16 * C2 || (cur_tight[t] + 1 < sLvNtight[tl[t]] && nh >= kEarlyHits)) {
        table_resolve(A, g, hw_warp_mem(wb, C2, t), lane, hbw + t * hcap, min(nh, hcap));
        anyhits[t] = true;
        __syncwarp();
        if (lane == 0) st_of(t)->nhits = 0;
        if (st_of(t)->B_valid) {
          const int B = st_of(t)->B;
          for (int q = sLvNtight[tl[t]] - 1; q > cur_tight[t]; --q) {
            if (sLvTau[tl[t]][1 + q] >= B) {
              cur_tight[t] = q;
              break;
            }
          }
        }
        __syncwarp();
      }
    }
    const int ct = half ? cur_tight[1] : cur_tight[0];
    ktab_me = reinterpret_cast<const uint4*>(sLvTab[lv_me][1 + ct]);  // ct = -1: the level's own table
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (tb[t] < 0) continue;
      const int bt = tb[t];
      const int route = A.route + tl[t];  // DTO_ROUTE_LEVEL0 + level
      const TableWarpMem mt = hw_warp_mem(wb, C2, t);
      const int nh = min(mt.st->nhits, hcap);
      if (nh > 0) table_resolve(A, g, mt, lane, hbw + t * hcap, nh);
      if ((nh > 0 || anyhits[t]) && mt.st->B_valid) {
        if (isinf(mt.st->bp)) {
          // no FP64 tail evaluated yet for this task: queue its survivors
          table_defer(A, g, mt, lane, bt, route);
        } else {
          table_refine(A, g, mt, lane);
          if (lane == 0) A.out[bt] = TaskResult{mt.st->bp, mt.st->bi, mt.st->bj, mt.st->bk, route};
        }
        tb[t] = -1;
      } else {
        // no cell reaches the level's bound: the next level takes the task
        // in this half-warp's next sweep, or after the last level the
        // exhaustive screen
        ++nfall;
        if (tl[t] + 1 < A.nlev) {
          tl[t] += 1;
        } else {
          if (lane == 0) A.fallback[atomicAdd(A.nfallback, 1)] = bt;
          tb[t] = -1;
        }
      }
      __syncwarp();
    }
  }
  if (st_of(0)->npend > 0) table_pending_flush(A, g, hw_warp_mem(wb, C2, 0), lane);
  if (lane == 0 && A.n_refined) {
    atomicAdd(A.n_refined, st_of(0)->n64);
    atomicAdd(A.n_refined + 1, st_of(0)->n32);
    atomicAdd(A.n_refined + 2, nfall);
  }
}

template <int C2, bool Multi>
cudaError_t launch_table_hw_kernel(const TableGridArgs& a, int ctas, size_t smem, cudaStream_t s) {
  cudaError_t e = raise_smem_limit((const void*)table_hw_kernel<C2, Multi>, smem);
  if (e != cudaSuccess) return e;
  table_hw_kernel<C2, Multi><<<ctas, kTableWarps * 32, smem, s>>>(a);
  return cudaGetLastError();
}

// The half-warp sweep of 2 C columns per lane: one pair, or several
// (segments) of the same C.
template <int C>
cudaError_t launch_table_grid_impl(const TableGridArgs& a, int ctas, size_t smem, cudaStream_t s) {
  if (a.segs) return launch_table_hw_kernel<2 * C, true>(a, ctas, smem, s);
  return launch_table_hw_kernel<2 * C, false>(a, ctas, smem, s);
}

}  // namespace dto

#define DTO_DEFINE_TABLE_GRID(CC)                                                                     \
  namespace dto {                                                                                     \
  cudaError_t launch_table_grid_c##CC(const TableGridArgs& a, int ctas, size_t smem, cudaStream_t s) { \
    return launch_table_grid_impl<CC>(a, ctas, smem, s);                                              \
  }                                                                                                   \
  }
