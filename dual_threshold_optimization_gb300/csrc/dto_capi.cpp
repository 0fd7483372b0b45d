// dto_capi.cpp -- host side of libdto.so: contexts, list pairs, batch
// orchestration of the permutation null, and the C ABI declared in
// include/dto.h.
//
// Host arithmetic that feeds the kernels (thresholds, the log-factorial
// tables) is written so that it gives the same bits on x86-64 and aarch64:
// only IEEE basic operations and explicit fma(), compiled with
// -ffp-contract=off.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/dto.h"
#include "dto_internal.h"

using namespace dto;

// Buffers of one in-flight batch of the table-screen pipeline.
struct BatchSlot {
  void* dX = nullptr;
  size_t xBytes = 0;
  void* dRes = nullptr;
  size_t resBytes = 0;
  void* hRes = nullptr;  // pinned
  size_t hResBytes = 0;
  void* dFall = nullptr;
  size_t fallBytes = 0;
  void* dIdx = nullptr;
  size_t idxBytes = 0;
  int* dCnt = nullptr;  // [0, 8): task counters, [8, 12): fallback counts
  cudaEvent_t ev[8] = {};  // perm start/end, tables start, -, exhaustive start/end, tables done, batch done
  bool busy = false;
  long long b0 = 0;
  int cnt = 0;
};

struct dto_ctx {
  int device = 0;
  int nsm = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // the unpermuted task runs here next to the first batch
  cudaEvent_t evSide = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t evk[4] = {nullptr, nullptr, nullptr, nullptr};  // perm start/end, grid start/end
  // per-call accounting (reset by dto_run)
  double acc_grid_ms = 0.0, acc_perm_ms = 0.0;
  long long acc_launches = 0, acc_h2d = 0, acc_d2h = 0;
  std::string err;
  std::mutex mu;
  // ln(m!) as double-double, m = 0..lf_cap
  long long lf_cap = -1;
  std::vector<double> lf_hi, lf_lo;
  double2* dLF = nullptr;
  // scratch, grown on demand
  void* dX = nullptr;
  size_t xBytes = 0;
  void* dSig = nullptr;
  size_t sigBytes = 0;
  void* dRes = nullptr;
  size_t resBytes = 0;
  void* hRes = nullptr;  // pinned
  size_t hResBytes = 0;
  int* dWork = nullptr;
  unsigned long long* dRefined = nullptr;
  unsigned* dGuess = nullptr;  // bound histogram shared by the batches of one run
  void* dHits[2] = {nullptr, nullptr};  // per-warp hit buffers of the table screen, one per stream
  size_t hitBytes[2] = {0, 0};
  BatchSlot slot[2];           // double-buffered batches of the table-screen pipeline
  int* dNFall = nullptr;
};

struct dto_pair {
  dto_ctx* ctx = nullptr;
  uint32_t pair_id = 0;
  long long N1 = 0, N2 = 0, npop = 0, nfeat = 0, ncommon = 0;
  bool same_set = false;
  std::vector<uint32_t> r1, r2, T1, T2;
  std::vector<int32_t> order1, order2, f1, f2;
  std::vector<int> c1, c2, map12;
  std::vector<int16_t> lab2, ylab;
  int C = 0, fshift = 0;
  long long upload_bytes = 0;  // host-to-device bytes of dto_pair_create
  // device
  int* dRow = nullptr;
  int* dNcnt = nullptr;
  uint32_t* dF = nullptr;
  int16_t* dYlab = nullptr;
  int16_t* dLab2 = nullptr;
  int* dMap12 = nullptr;
  uint16_t* dKthr[3] = {nullptr, nullptr, nullptr};  // table screens, built for bounds kthr_tau
  int kthr_tau[3] = {0, 0, 0};
  bool kthr_ok[3] = {false, false, false};
  PairDev dev{};
};

namespace {

// ---------------------------------------------------------------------------
// Double-double helpers for the log-factorial table (same specification as the
// device code; Dekker 1971, Knuth TAOCP 4.2.2).
// ---------------------------------------------------------------------------
struct DD {
  double hi, lo;
};
inline DD h_two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline DD h_fast_two_sum(double a, double b) {
  double s = a + b;
  return {s, b - (s - a)};
}
inline DD h_add(DD x, DD y) {
  DD s = h_two_sum(x.hi, y.hi), t = h_two_sum(x.lo, y.lo);
  double e = s.lo + t.hi;
  DD u = h_fast_two_sum(s.hi, e);
  e = u.lo + t.lo;
  return h_fast_two_sum(u.hi, e);
}
inline DD h_mul(DD x, DD y) {
  double p = x.hi * y.hi;
  double e = std::fma(x.hi, y.hi, -p);
  e = std::fma(x.hi, y.lo, e);
  e = std::fma(x.lo, y.hi, e);
  return h_fast_two_sum(p, e);
}
inline DD h_div_int(DD x, double d) {
  double q1 = x.hi / d;
  double r = std::fma(-q1, d, x.hi);
  r = r + x.lo;
  double q2 = r / d;
  return h_fast_two_sum(q1, q2);
}

// ln(m!) for m = 0..nmax: ln(m) = ln(m-1) + 2 atanh(1/(2m-1)), the atanh
// Taylor series summed until a term is below 2^-110 of the sum.
void lf_table_dd(long long nmax, std::vector<double>& hi, std::vector<double>& lo) {
  hi.assign((size_t)nmax + 1, 0.0);
  lo.assign((size_t)nmax + 1, 0.0);
  DD lf{0.0, 0.0}, ln{0.0, 0.0};
  for (long long m = 2; m <= nmax; ++m) {
    DD s = h_div_int(DD{1.0, 0.0}, (double)(2 * m - 1));
    DD s2 = h_mul(s, s), pw = s, sum = s;
    for (long long i = 1; i < 200; ++i) {
      pw = h_mul(pw, s2);
      DD term = h_div_int(pw, (double)(2 * i + 1));
      sum = h_add(sum, term);
      if (std::fabs(term.hi) < std::ldexp(std::fabs(sum.hi), -110)) break;
    }
    ln = h_add(ln, DD{2.0 * sum.hi, 2.0 * sum.lo});
    lf = h_add(lf, ln);
    hi[(size_t)m] = lf.hi;
    lo[(size_t)m] = lf.lo;
  }
}

// round(x * 2^f) of a double-double x, to the nearest integer.
long long dd_round_scaled(double hi, double lo, int f) {
  double x = std::ldexp(hi, f), y = std::ldexp(lo, f);
  double r = std::nearbyint(x);
  double frac = (x - r) + y;
  if (frac > 0.5) r += 1.0;
  else if (frac < -0.5) r -= 1.0;
  return (long long)r;
}

int set_err(dto_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_err(dto_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_err(ctx, e == cudaErrorMemoryAllocation ? DTO_ERR_OOM : DTO_ERR_CUDA, m);
}

#define CK(call)                                     \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_err(ctx, e_, #call); \
  } while (0)

int grow(dto_ctx* ctx, void** p, size_t* cap, size_t need) {
  if (need <= *cap) return DTO_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t sz = std::max(need, (size_t)4096);
  CK(cudaMalloc(p, sz));
  *cap = sz;
  return DTO_OK;
}

int grow_host(dto_ctx* ctx, void** p, size_t* cap, size_t need) {
  if (need <= *cap) return DTO_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  size_t sz = std::max(need, (size_t)4096);
  CK(cudaMallocHost(p, sz));
  *cap = sz;
  return DTO_OK;
}

int ensure_lf(dto_ctx* ctx, long long nmax) {
  if (nmax <= ctx->lf_cap) return DTO_OK;
  long long cap = std::max(nmax, 2 * ctx->lf_cap);
  cap = std::max(cap, 1024LL);
  lf_table_dd(cap, ctx->lf_hi, ctx->lf_lo);
  std::vector<double2> h((size_t)cap + 1);
  for (size_t m = 0; m <= (size_t)cap; ++m) h[m] = make_double2(ctx->lf_hi[m], ctx->lf_lo[m]);
  if (ctx->dLF) cudaFree(ctx->dLF);
  ctx->dLF = nullptr;
  ctx->lf_cap = -1;
  CK(cudaMalloc(&ctx->dLF, h.size() * sizeof(double2)));
  CK(cudaMemcpy(ctx->dLF, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
  ctx->lf_cap = cap;
  return DTO_OK;
}

std::vector<uint32_t> thresholds_of(uint32_t max_rank) {
  std::vector<uint32_t> t;
  uint32_t cur = 1;
  while (cur <= max_rank) {
    t.push_back(cur);
    double nx = std::floor((double)cur * 1.01 + 1.0);
    if (nx >= 4294967296.0) break;
    cur = (uint32_t)nx;
  }
  return t;
}

constexpr int kCs[] = {4, 8, 12, 16, 20, 24, 28, 32};

// Quantile of the first batch's minimum p-values that sets the level-0 table.
#ifndef DTO_L0_QUANTILE
#define DTO_L0_QUANTILE 0.90
#endif
constexpr double kLevel0Quantile = DTO_L0_QUANTILE;

int pick_C(int n2) {
  for (int c : kCs)
    if (32 * c >= n2) return c;
  return -1;
}

// Rows of the grid kernel need 16-byte aligned starts for vector loads.
long long xstride_of(long long N1) { return (N1 + 7) & ~7LL; }

int check_perm(const int32_t* idx, long long L) {
  std::vector<char> seen((size_t)L, 0);
  for (long long p = 0; p < L; ++p) {
    int32_t v = idx[p];
    if (v < 0 || v >= L || seen[(size_t)v]) return 0;
    seen[(size_t)v] = 1;
  }
  return 1;
}

void fill_result(const dto_pair* P, const TaskResult& r, int permuted, dto_result* o) {
  o->rank1 = P->T1[(size_t)r.i];
  o->rank2 = P->T2[(size_t)r.j];
  o->set1_len = P->c1[(size_t)r.i];
  o->set2_len = P->c2[(size_t)r.j];
  o->population_size = P->npop;
  o->intersection_size = r.k;
  o->pvalue = r.p;
  o->permuted = permuted;
  o->i = r.i;
  o->j = r.j;
  o->status = r.status;
}

int grid_tasks(dto_ctx* ctx, dto_pair* P, const int16_t* dX, long long xstride, int ntask, int mode,
               TaskResult* dOut, int* dumpK = nullptr, double* dumpP = nullptr, bool guess = false,
               cudaStream_t stream = nullptr) {
  if (!stream) stream = ctx->stream;
  GridArgs a{};
  a.P = P->dev;
  a.P.LF = ctx->dLF;  // the context's table may have grown since the pair was created
  a.X = dX;
  a.xstride = xstride;
  a.ntask = ntask;
  a.mode = mode;
  size_t smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1);
  a.smemF = smemF <= ctx->smem_optin ? 1 : 0;
  a.out = dOut;
  a.work = ctx->dWork;
  a.n_refined = ctx->dRefined;
  a.guess_hist = (guess && mode == kModeScreen) ? ctx->dGuess : nullptr;
  a.dump_k = dumpK;
  a.dump_p = dumpP;
  CK(cudaMemsetAsync(ctx->dWork, 0, sizeof(int), stream));
  int ctas = std::min(ctx->nsm, (ntask + kGridWarps - 1) / kGridWarps);
  ctas = std::max(ctas, 1);
  CK(cudaEventRecord(ctx->evk[2], stream));
  CK(launch_grid(a, ctas, stream));
  CK(cudaEventRecord(ctx->evk[3], stream));
  ctx->acc_launches += 1;
  return DTO_OK;
}

// Table screen `level` for bound tau (fixed-point ln p), built on the device.
int ensure_table(dto_ctx* ctx, dto_pair* P, int level, int tau) {
  if (P->kthr_ok[level] && P->kthr_tau[level] == tau) return DTO_OK;
  if (!P->dKthr[level]) CK(cudaMalloc(&P->dKthr[level], table_entries(P->C, P->dev.n1) * 2));
  TableArgs t{};
  t.n1 = P->dev.n1;
  t.n2 = P->dev.n2;
  t.N = (int)P->npop;
  t.C = P->C;
  t.rowstart = P->dRow;
  t.ncnt = P->dNcnt;
  t.F = P->dF;
  t.fshift = P->fshift;
  t.tau = tau;
  t.packed = P->ncommon <= kPackedMaxCommon ? 1 : 0;
  t.kthr = P->dKthr[level];
  CK(launch_table_build(t, ctx->nsm, ctx->stream));
  ctx->acc_launches += 1;
  P->kthr_tau[level] = tau;
  P->kthr_ok[level] = true;
  return DTO_OK;
}

// Tasks [0, ntask) of X through the table ladder: level l takes the tasks
// that level l-1 could not settle (their minimum lies above its bound), and
// the exhaustive screen takes what the last level leaves.  The lists and
// their counts stay on the device.  `fall` holds nlev lists of cap entries,
// `cnts` 8 task counters then 4 list counts.  The levels run on the context's
// stream; the exhaustive screen runs on `xstream` after `evTab` (which may be
// the same stream).
int table_levels(dto_ctx* ctx, dto_pair* P, const int16_t* X, long long xstride, int ntask, TaskResult* dOut,
                 int lev_begin, int lev_end, int* fall, int* cnts, cudaStream_t stream, int hb) {
  const int cap = std::max(ntask, 1);
  const int hitcap = 8192;
  int rc = grow(ctx, &ctx->dHits[hb], &ctx->hitBytes[hb], (size_t)kTableCtasPerSm * ctx->nsm * kTableWarps * hitcap * 8);
  if (rc) return rc;
  if (lev_begin == 0) CK(cudaMemsetAsync(cnts, 0, 12 * sizeof(int), stream));
  for (int level = lev_begin; level < lev_end; ++level) {
    TableGridArgs a{};
    a.P = P->dev;
    a.P.LF = ctx->dLF;
    a.X = X;
    a.xstride = xstride;
    a.ntask = ntask;
    a.tau = P->kthr_tau[level];
    a.kthr = P->dKthr[level];
    a.packed = P->ncommon <= kPackedMaxCommon ? 1 : 0;
    a.out = dOut;
    a.work = cnts + level;
    a.n_refined = ctx->dRefined;
    a.fallback = fall + (size_t)level * cap;
    a.nfallback = cnts + 8 + level;
    a.task_list = level == 0 ? nullptr : fall + (size_t)(level - 1) * cap;
    a.ntask_dev = level == 0 ? nullptr : cnts + 8 + level - 1;
    a.hitbuf = (int2*)ctx->dHits[hb];
    a.hitcap = hitcap;
    // a later level sees the tasks the earlier ones left (about 10 % and 1 %
    // of the batch); one warp per expected task keeps its latency to one sweep
    const double expect = level == 0 ? 1.0 : level == 1 ? 0.15 : 0.03;
    const int want = (int)(expect * (double)ntask / kTableWarps) + 1;
    const int ctas = std::max(1, std::min(kTableCtasPerSm * ctx->nsm, want));
    CK(launch_table_grid(a, P->C, ctas, stream));
  }
  ctx->acc_launches += lev_end - lev_begin;
  return DTO_OK;
}

// The exhaustive screen of what the last table level left, on `stream`.
int table_exhaustive(dto_ctx* ctx, dto_pair* P, const int16_t* X, long long xstride, int ntask, TaskResult* dOut,
                     int nlev, const int* fall, int* cnts, cudaStream_t stream) {
  const int cap = std::max(ntask, 1);
  GridArgs g{};
  g.P = P->dev;
  g.P.LF = ctx->dLF;
  g.X = X;
  g.xstride = xstride;
  g.ntask = ntask;
  g.mode = kModeScreen;
  g.smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1) <= ctx->smem_optin ? 1 : 0;
  g.out = dOut;
  g.work = cnts + nlev;
  g.n_refined = ctx->dRefined;
  g.task_list = fall + (size_t)(nlev - 1) * cap;
  g.ntask_dev = cnts + 8 + nlev - 1;
  CK(launch_grid(g, ctx->nsm, stream));
  ctx->acc_launches += 1;
  return DTO_OK;
}

int fixed_log(double p, int fshift) {
  double t = std::floor(std::log(p) * std::ldexp(1.0, fshift));
  return (int)std::max(-2.0e9, std::min(0.0, t));
}

// Labels of n_perm permutations starting at perm id `first` into ctx->dX.
int make_labels_launch(dto_ctx* ctx, dto_pair* P, uint64_t seed, uint32_t first, int count,
                       const int32_t* dIdx, int16_t* X, long long xs);

int make_labels(dto_ctx* ctx, dto_pair* P, uint64_t seed, uint32_t first, int count,
                const int32_t* dIdx /* nullable: test mode, [count][N1+N2] */, int row0 = 0) {
  long long xs = xstride_of(P->N1);
  int rc = grow(ctx, &ctx->dX, &ctx->xBytes, (size_t)(count + row0) * xs * 2);
  if (rc) return rc;
  int16_t* X = (int16_t*)ctx->dX + (size_t)row0 * xs;
  CK(cudaEventRecord(ctx->evk[0], ctx->stream));
  rc = make_labels_launch(ctx, P, seed, first, count, dIdx, X, xs);
  CK(cudaEventRecord(ctx->evk[1], ctx->stream));
  return rc;
}

int make_labels_launch(dto_ctx* ctx, dto_pair* P, uint64_t seed, uint32_t first, int count,
                       const int32_t* dIdx, int16_t* X, long long xs) {
  int rc = DTO_OK;
  if (dIdx) {
    ComposeArgs c{};
    c.N1 = (int)P->N1;
    c.N2 = (int)P->N2;
    c.idx1 = dIdx;
    c.idx2 = dIdx + P->N1;
    c.stride = P->N1 + P->N2;
    c.map12 = P->dMap12;
    c.lab2 = P->dLab2;
    c.X = X;
    c.xstride = xs;
    CK(launch_compose(c, count, ctx->stream));
    ctx->acc_launches += 1;
    return DTO_OK;
  }
  PermArgs a{};
  a.seed = seed;
  a.pair_id = P->pair_id;
  a.perm_base = first;
  a.xstride = xs;
  if (P->same_set) {
    // With identical feature sets only the relative order of the two lists
    // matters: list 1 is shuffled, list 2 kept (idx2 = identity).
    a.L = (int)P->N1;
    a.list_tag = 1;
    a.Ylab = P->dYlab;
    a.X = X;
    CK(launch_perm(a, count, ctx->stream));
    ctx->acc_launches += 1;
    return DTO_OK;
  }
  long long ss = P->N1 + P->N2;
  rc = grow(ctx, &ctx->dSig, &ctx->sigBytes, (size_t)count * ss * 4);
  if (rc) return rc;
  int* sig = (int*)ctx->dSig;
  a.L = (int)P->N1;
  a.list_tag = 1;
  a.sigma = sig;
  a.sstride = ss;
  CK(launch_perm(a, count, ctx->stream));
  a.L = (int)P->N2;
  a.list_tag = 2;
  a.sigma = sig + P->N1;
  CK(launch_perm(a, count, ctx->stream));
  ComposeArgs c{};
  c.N1 = (int)P->N1;
  c.N2 = (int)P->N2;
  c.idx1 = sig;
  c.idx2 = sig + P->N1;
  c.stride = ss;
  c.map12 = P->dMap12;
  c.lab2 = P->dLab2;
  c.X = X;
  c.xstride = xs;
  CK(launch_compose(c, count, ctx->stream));
  ctx->acc_launches += 3;
  return DTO_OK;
}

}  // namespace

extern "C" {

int dto_version(void) { return 10000; }

const char* dto_status_string(int s) {
  switch (s) {
    case DTO_OK: return "ok";
    case DTO_ERR_INVALID: return "invalid argument";
    case DTO_ERR_OOM: return "out of memory";
    case DTO_ERR_TIMEOUT: return "timeout";
    case DTO_ERR_CUDA: return "CUDA error";
    case DTO_ERR_NOT_FOUND: return "not found";
    default: return "unknown status";
  }
}

int dto_ctx_create(int device, dto_ctx** out) {
  if (!out) return DTO_ERR_INVALID;
  *out = nullptr;
  dto_ctx* ctx = new dto_ctx();
  ctx->device = device;
  auto fail = [&](cudaError_t e) {
    delete ctx;
    return e == cudaErrorMemoryAllocation ? DTO_ERR_OOM : DTO_ERR_CUDA;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(e);
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) return fail(e);
  ctx->nsm = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&ctx->evSide, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&ctx->ev0)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&ctx->ev1)) != cudaSuccess) return fail(e);
  for (int q = 0; q < 4; ++q)
    if ((e = cudaEventCreate(&ctx->evk[q])) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&ctx->dWork, 256)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&ctx->dRefined, 256)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&ctx->dGuess, 2048)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&ctx->dNFall, 256)) != cudaSuccess) return fail(e);
  *out = ctx;
  return DTO_OK;
}

int dto_ctx_destroy(dto_ctx* ctx) {
  if (!ctx) return DTO_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->side) cudaStreamSynchronize(ctx->side);
  cudaFree(ctx->dLF);
  cudaFree(ctx->dX);
  cudaFree(ctx->dSig);
  cudaFree(ctx->dRes);
  cudaFreeHost(ctx->hRes);
  cudaFree(ctx->dWork);
  cudaFree(ctx->dRefined);
  cudaFree(ctx->dGuess);
  cudaFree(ctx->dHits[0]);
  cudaFree(ctx->dHits[1]);
  for (BatchSlot& sl : ctx->slot) {
    cudaFree(sl.dX);
    cudaFree(sl.dRes);
    cudaFreeHost(sl.hRes);
    cudaFree(sl.dFall);
    cudaFree(sl.dIdx);
    cudaFree(sl.dCnt);
    for (cudaEvent_t e : sl.ev)
      if (e) cudaEventDestroy(e);
  }
  cudaFree(ctx->dNFall);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (int q = 0; q < 4; ++q)
    if (ctx->evk[q]) cudaEventDestroy(ctx->evk[q]);
  if (ctx->evSide) cudaEventDestroy(ctx->evSide);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return DTO_OK;
}

const char* dto_last_error(const dto_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* dto_ctx_stream(dto_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int64_t dto_generate_thresholds(uint32_t max_rank, uint32_t* out, int64_t cap) {
  std::vector<uint32_t> t = thresholds_of(max_rank);
  for (size_t q = 0; q < t.size() && (int64_t)q < cap; ++q) out[q] = t[q];
  return (int64_t)t.size();
}

double dto_fdr(int64_t l1, int64_t l2, int64_t overlap, int64_t population, double sensitivity) {
  double df = std::max((double)overlap / sensitivity, 0.0);
  double bm = std::max((double)l1 - df, 0.0), rm = std::max((double)l2 - df, 0.0);
  double den = (double)population * (double)overlap;
  return den > 0.0 ? (bm * rm) / den : 0.0;
}

int dto_pair_create(dto_ctx* ctx, const uint32_t* ranks1, const int32_t* feat1, int64_t n1,
                    const uint32_t* ranks2, const int32_t* feat2, int64_t n2, int64_t n_features,
                    int64_t population, dto_pair** out) {
  if (!ctx || !out) return DTO_ERR_INVALID;
  std::lock_guard<std::mutex> g(ctx->mu);
  *out = nullptr;
  if (n1 <= 0 || n2 <= 0 || !ranks1 || !ranks2 || !feat1 || !feat2)
    return set_err(ctx, DTO_ERR_INVALID, "empty ranked feature list");
  if (n1 > kMaxListLen || n2 > kMaxListLen)
    return set_err(ctx, DTO_ERR_INVALID, "ranked feature lists are limited to 65534 features");
  if (population <= 0 || population > 4000000)
    return set_err(ctx, DTO_ERR_INVALID, "population size must lie in [1, 4000000]");
  if (n_features <= 0) return set_err(ctx, DTO_ERR_INVALID, "n_features must be positive");
  CK(cudaSetDevice(ctx->device));
  dto_pair* P = new dto_pair();
  P->ctx = ctx;
  P->pair_id = 0;  // Philox stream id; dto_pair_set_stream changes it
  P->N1 = n1;
  P->N2 = n2;
  P->npop = population;
  P->nfeat = n_features;
  // stable sort by rank (src/collections/ranked.rs:527-542)
  auto sort_list = [](const uint32_t* r, int64_t n, std::vector<int32_t>& order) {
    order.resize((size_t)n);
    for (int64_t q = 0; q < n; ++q) order[(size_t)q] = (int32_t)q;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return r[a] < r[b]; });
  };
  sort_list(ranks1, n1, P->order1);
  sort_list(ranks2, n2, P->order2);
  P->r1.resize((size_t)n1);
  P->f1.resize((size_t)n1);
  P->r2.resize((size_t)n2);
  P->f2.resize((size_t)n2);
  std::vector<int> pos2((size_t)n_features, -1), pos1((size_t)n_features, -1);
  for (int64_t p = 0; p < n1; ++p) {
    int32_t q = P->order1[(size_t)p];
    P->r1[(size_t)p] = ranks1[q];
    int32_t f = feat1[q];
    if (f < 0 || f >= n_features) { delete P; return set_err(ctx, DTO_ERR_INVALID, "feature id out of range in list 1"); }
    if (pos1[(size_t)f] >= 0) { delete P; return set_err(ctx, DTO_ERR_INVALID, "duplicate feature id in list 1"); }
    pos1[(size_t)f] = (int)p;
    P->f1[(size_t)p] = f;
  }
  for (int64_t p = 0; p < n2; ++p) {
    int32_t q = P->order2[(size_t)p];
    P->r2[(size_t)p] = ranks2[q];
    int32_t f = feat2[q];
    if (f < 0 || f >= n_features) { delete P; return set_err(ctx, DTO_ERR_INVALID, "feature id out of range in list 2"); }
    if (pos2[(size_t)f] >= 0) { delete P; return set_err(ctx, DTO_ERR_INVALID, "duplicate feature id in list 2"); }
    pos2[(size_t)f] = (int)p;
    P->f2[(size_t)p] = f;
  }
  P->T1 = thresholds_of(P->r1.back());
  P->T2 = thresholds_of(P->r2.back());
  if (P->T1.empty() || P->T2.empty()) {
    delete P;
    return set_err(ctx, DTO_ERR_INVALID, "a list has no thresholds (maximum rank is 0)");
  }
  const int nt1 = (int)P->T1.size(), nt2 = (int)P->T2.size();
  P->C = pick_C(nt2);
  if (P->C < 0 || nt1 >= 32768) {
    delete P;
    return set_err(ctx, DTO_ERR_INVALID, "threshold grid too large (at most 1024 list-2 thresholds)");
  }
  // set sizes c(t) = #{rank <= t} (permutation independent)
  P->c1.resize((size_t)nt1);
  P->c2.resize((size_t)nt2);
  for (int i = 0, p = 0; i < nt1; ++i) { while (p < n1 && P->r1[(size_t)p] <= P->T1[(size_t)i]) ++p; P->c1[(size_t)i] = p; }
  for (int j = 0, p = 0; j < nt2; ++j) { while (p < n2 && P->r2[(size_t)p] <= P->T2[(size_t)j]) ++p; P->c2[(size_t)j] = p; }
  if (P->c1.back() > population || P->c2.back() > population) {
    delete P;
    return set_err(ctx, DTO_ERR_INVALID, "Failed to create hypergeometric distribution: set size exceeds the population size");
  }
  // labels of list-2 positions
  const int Cp = P->C | 1;
  P->lab2.assign((size_t)n2, -1);
  for (int64_t p = 0, j = 0; p < n2; ++p) {
    while (j < nt2 && P->T2[(size_t)j] < P->r2[(size_t)p]) ++j;
    if (j < nt2) P->lab2[(size_t)p] = (int16_t)((j / P->C) * Cp + (j % P->C));
  }
  P->map12.assign((size_t)n1, -1);
  P->ylab.assign((size_t)n1, -1);
  long long common = 0;
  for (int64_t p = 0; p < n1; ++p) {
    int q = pos2[(size_t)P->f1[(size_t)p]];
    P->map12[(size_t)p] = q;
    if (q >= 0) { ++common; P->ylab[(size_t)p] = P->lab2[(size_t)q]; }
  }
  P->ncommon = common;
  P->same_set = (common == n1 && common == n2);
  // fixed-point fraction bits: |ln pmf| <= N ln 2 must fit in int32 with slack
  int f = 0;
  while (f < 24 && ((double)population * 0.6931471805599453 + 64.0) * std::ldexp(1.0, f + 1) < 2.0e9) ++f;
  P->fshift = f;
  int rc = ensure_lf(ctx, population);
  if (rc) { delete P; return rc; }
  std::vector<uint32_t> F((size_t)population + 1);
  for (long long m = 0; m <= population; ++m)
    F[(size_t)m] = (uint32_t)(unsigned long long)dd_round_scaled(ctx->lf_hi[(size_t)m], ctx->lf_lo[(size_t)m], f);
  std::vector<int> row((size_t)nt1 + 1);
  row[0] = 0;
  for (int i = 0; i < nt1; ++i) row[(size_t)i + 1] = P->c1[(size_t)i];
  auto up = [&](void** d, const void* h, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(d, std::max(bytes, (size_t)16));
    if (e != cudaSuccess) return e;
    P->upload_bytes += (long long)bytes;
    return cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = up((void**)&P->dRow, row.data(), row.size() * 4);
  if (e == cudaSuccess) e = up((void**)&P->dNcnt, P->c2.data(), P->c2.size() * 4);
  if (e == cudaSuccess) e = up((void**)&P->dF, F.data(), F.size() * 4);
  if (e == cudaSuccess) e = up((void**)&P->dYlab, P->ylab.data(), P->ylab.size() * 2);
  if (e == cudaSuccess) e = up((void**)&P->dLab2, P->lab2.data(), P->lab2.size() * 2);
  if (e == cudaSuccess) e = up((void**)&P->dMap12, P->map12.data(), P->map12.size() * 4);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    dto_pair_destroy(P);
    return cuda_err(ctx, e, "pair upload");
  }
  PairDev& d = P->dev;
  d.n1 = nt1;
  d.n2 = nt2;
  d.N1 = (int)n1;
  d.N2 = (int)n2;
  d.Npop = population;
  d.C = P->C;
  d.fshift = f;
  d.rowstart = P->dRow;
  d.ncnt = P->dNcnt;
  d.F = P->dF;
  d.LF = nullptr;  // bound at launch: the context's table can be reallocated
  d.Ylab = P->dYlab;
  d.lab2 = P->dLab2;
  d.map12 = P->dMap12;
  *out = P;
  return DTO_OK;
}

int dto_pair_destroy(dto_pair* P) {
  if (!P) return DTO_ERR_INVALID;
  cudaFree(P->dRow);
  cudaFree(P->dNcnt);
  cudaFree(P->dF);
  cudaFree(P->dYlab);
  cudaFree(P->dLab2);
  cudaFree(P->dMap12);
  for (int l = 0; l < 3; ++l) cudaFree(P->dKthr[l]);
  delete P;
  return DTO_OK;
}

int dto_pair_info(const dto_pair* P, int64_t* nt1, int64_t* nt2, int64_t* ncommon) {
  if (!P) return DTO_ERR_INVALID;
  if (nt1) *nt1 = (int64_t)P->T1.size();
  if (nt2) *nt2 = (int64_t)P->T2.size();
  if (ncommon) *ncommon = P->ncommon;
  return DTO_OK;
}

int dto_pair_thresholds(const dto_pair* P, uint32_t* t1, uint32_t* t2) {
  if (!P) return DTO_ERR_INVALID;
  if (t1) std::copy(P->T1.begin(), P->T1.end(), t1);
  if (t2) std::copy(P->T2.begin(), P->T2.end(), t2);
  return DTO_OK;
}

int64_t dto_pair_upload_bytes(const dto_pair* P) { return P ? (int64_t)P->upload_bytes : -1; }

int dto_pair_set_stream(dto_pair* P, uint32_t stream_id) {
  if (!P) return DTO_ERR_INVALID;
  P->pair_id = stream_id;
  return DTO_OK;
}

int dto_pair_order(const dto_pair* P, int32_t* o1, int32_t* o2) {
  if (!P) return DTO_ERR_INVALID;
  if (o1) std::copy(P->order1.begin(), P->order1.end(), o1);
  if (o2) std::copy(P->order2.begin(), P->order2.end(), o2);
  return DTO_OK;
}

int dto_run(dto_ctx* ctx, dto_pair* P, int64_t n_perm, uint64_t seed, const int32_t* perm_idx,
            int precision, dto_result* out_unpermuted, double* out_minp, dto_result* out_perm,
            dto_summary* out_summary) {
  return dto_run_range(ctx, P, 1u, n_perm, seed, perm_idx, precision, out_unpermuted, out_minp,
                       out_perm, out_summary);
}

int dto_run_range(dto_ctx* ctx, dto_pair* P, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                  const int32_t* perm_idx, int precision, dto_result* out_unpermuted, double* out_minp,
                  dto_result* out_perm, dto_summary* out_summary) {
  if (!ctx || !P || P->ctx != ctx || !out_unpermuted) return set_err(ctx, DTO_ERR_INVALID, "null argument");
  if (n_perm < 0 || n_perm > 0x7fffffffLL || (long long)perm_first + n_perm > 0xffffffffLL)
    return set_err(ctx, DTO_ERR_INVALID, "n_perm out of range");
  if (precision != DTO_PRECISION_FP64 && precision != DTO_PRECISION_SCREEN)
    return set_err(ctx, DTO_ERR_INVALID, "unknown precision");
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  const long long L12 = P->N1 + P->N2;
  if (perm_idx) {
    for (long long b = 0; b < n_perm; ++b) {
      if (!check_perm(perm_idx + b * L12, P->N1) || !check_perm(perm_idx + b * L12 + P->N1, P->N2))
        return set_err(ctx, DTO_ERR_INVALID, "perm_idx row is not a permutation");
    }
  }
  const int mode = precision == DTO_PRECISION_FP64 ? kModeFull64 : kModeScreen;
  const long long xs = xstride_of(P->N1);
  // batch size: bounded by 1 GiB of labels (and of test-mode indices)
  long long batch = std::max(1LL, std::min<long long>((1LL << 30) / (xs * 2), 1LL << 20));
  if (perm_idx) batch = std::min(batch, std::max(1LL, (1LL << 30) / (L12 * 4)));
  if (!P->same_set && !perm_idx) batch = std::min(batch, std::max(1LL, (1LL << 30) / (L12 * 4)));
  batch = std::min<long long>(batch, std::max<long long>(n_perm, 1));
  int rc = grow(ctx, &ctx->dRes, &ctx->resBytes, (size_t)(batch + 1) * sizeof(TaskResult));
  if (rc) return rc;
  rc = grow_host(ctx, &ctx->hRes, &ctx->hResBytes, (size_t)(batch + 1) * sizeof(TaskResult));
  if (rc) return rc;
  void* dIdx = nullptr;
  size_t idxBytes = 0;
  struct Guard { void*& p; ~Guard() { if (p) cudaFree(p); } } guard{dIdx};
  TaskResult* dRes = (TaskResult*)ctx->dRes;
  TaskResult* hRes = (TaskResult*)ctx->hRes;
  ctx->acc_grid_ms = ctx->acc_perm_ms = 0.0;
  ctx->acc_launches = ctx->acc_h2d = ctx->acc_d2h = 0;
  CK(cudaMemsetAsync(ctx->dRefined, 0, 3 * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dGuess, 0, 2048, ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  std::vector<double> minp((size_t)n_perm);
  TaskResult unperm{};
  // The unpermuted task (task 0) rides in row 0 of the first batch, through
  // the exhaustive screen.  With the table screen (long runs), the first
  // batch holds first_batch permutations; its 90th and 99th percentiles and
  // maximum of the minimum p set the three-level table ladder of the
  // remaining batches.
  const long long first_batch = 1024;
  const bool use_table = (mode == kModeScreen) && n_perm > 2 * first_batch;
  auto take = [&](const TaskResult* hr, long long b0, int cnt) {
    for (int q = 0; q < cnt; ++q) {
      const TaskResult& r = hr[q];
      minp[(size_t)(b0 + q)] = r.p;
      if (out_minp) out_minp[b0 + q] = r.p;
      if (out_perm) fill_result(P, r, 1, &out_perm[b0 + q]);
    }
  };
  auto upload_idx = [&](void** buf, size_t* cap, long long b0, int cnt, const int32_t** dI) -> int {
    *dI = nullptr;
    if (!perm_idx || cnt <= 0) return DTO_OK;
    const size_t bytes = (size_t)cnt * L12 * 4;
    int r = grow(ctx, buf, cap, bytes);
    if (r) return r;
    CK(cudaMemcpyAsync(*buf, perm_idx + b0 * L12, bytes, cudaMemcpyHostToDevice, ctx->stream));
    ctx->acc_h2d += (long long)bytes;
    *dI = (const int32_t*)*buf;
    return DTO_OK;
  };
  if (!use_table) {
    for (long long b0 = 0; b0 < std::max<long long>(n_perm, 1); b0 += batch) {
      const int row0 = (b0 == 0) ? 1 : 0;
      const int cnt = (int)std::max(0LL, std::min(batch, n_perm - b0));
      const int32_t* dI = nullptr;
      rc = upload_idx(&dIdx, &idxBytes, b0, cnt, &dI);
      if (rc) return rc;
      if (cnt > 0) {
        rc = make_labels(ctx, P, seed, (uint32_t)(perm_first + b0), cnt, dI, row0);
        if (rc) return rc;
      } else {
        rc = grow(ctx, &ctx->dX, &ctx->xBytes, (size_t)xs * 2);
        if (rc) return rc;
      }
      if (row0) CK(cudaMemcpyAsync(ctx->dX, P->dYlab, (size_t)P->N1 * 2, cudaMemcpyDeviceToDevice, ctx->stream));
      const int ntask = cnt + row0;
      rc = grid_tasks(ctx, P, (const int16_t*)ctx->dX, xs, ntask, mode, dRes, nullptr, nullptr, true);
      if (rc) return rc;
      CK(cudaMemcpyAsync(hRes, dRes, (size_t)ntask * sizeof(TaskResult), cudaMemcpyDeviceToHost, ctx->stream));
      ctx->acc_d2h += (long long)ntask * (long long)sizeof(TaskResult);
      CK(cudaStreamSynchronize(ctx->stream));
      float ms = 0.f;
      if (cnt > 0 && cudaEventElapsedTime(&ms, ctx->evk[0], ctx->evk[1]) == cudaSuccess) ctx->acc_perm_ms += ms;
      if (cudaEventElapsedTime(&ms, ctx->evk[2], ctx->evk[3]) == cudaSuccess) ctx->acc_grid_ms += ms;
      if (row0) unperm = hRes[0];
      take(hRes + row0, b0, cnt);
    }
  } else {
    // Slots left busy by a call that returned early hold nothing of this call.
    CK(cudaStreamSynchronize(ctx->side));
    for (BatchSlot& sl : ctx->slot) sl.busy = false;
    // Batch 0 (task 0 + first_batch permutations) runs through the exhaustive
    // screen on the side stream.  Its slowest tasks (the permutations with
    // the largest minimum p) take several times a typical task; meanwhile the
    // main stream draws the labels of the first two pipelined batches.
    const int cnt0 = (int)first_batch;
    const int32_t* dI0 = nullptr;
    rc = upload_idx(&dIdx, &idxBytes, 0, cnt0, &dI0);
    if (rc) return rc;
    rc = make_labels(ctx, P, seed, perm_first, cnt0, dI0, 1);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->dX, P->dYlab, (size_t)P->N1 * 2, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->evSide, ctx->stream));
    CK(cudaStreamWaitEvent(ctx->side, ctx->evSide, 0));
    rc = grid_tasks(ctx, P, (const int16_t*)ctx->dX, xs, cnt0 + 1, mode, dRes, nullptr, nullptr, true, ctx->side);
    if (rc) return rc;
    CK(cudaMemcpyAsync(hRes, dRes, (size_t)(cnt0 + 1) * sizeof(TaskResult), cudaMemcpyDeviceToHost, ctx->side));
    ctx->acc_d2h += (long long)(cnt0 + 1) * (long long)sizeof(TaskResult);
    CK(cudaEventRecord(ctx->evSide, ctx->side));
    // Labels of the pipelined batches b = 0, 1, ... (permutations
    // first_batch + b * batch on), slot b & 1; the first two are drawn now.
    const long long pipe_from = first_batch;
    const long long npipe = (n_perm - pipe_from + batch - 1) / batch;
    bool drawn[2] = {false, false};
    auto draw = [&](long long it) -> int {
      BatchSlot& sl = ctx->slot[it & 1];
      const long long b0 = pipe_from + it * batch;
      const int cnt = (int)std::min(batch, n_perm - b0);
      if (!sl.ev[0])
        for (cudaEvent_t& e : sl.ev) CK(cudaEventCreate(&e));
      if (!sl.dCnt) CK(cudaMalloc(&sl.dCnt, 256));
      int r = grow(ctx, &sl.dX, &sl.xBytes, (size_t)cnt * xs * 2);
      if (!r) r = grow(ctx, &sl.dRes, &sl.resBytes, (size_t)cnt * sizeof(TaskResult));
      if (!r) r = grow_host(ctx, &sl.hRes, &sl.hResBytes, (size_t)cnt * sizeof(TaskResult));
      if (!r) r = grow(ctx, &sl.dFall, &sl.fallBytes, (size_t)3 * cnt * 4);
      if (r) return r;
      const int32_t* dI = nullptr;
      r = upload_idx(&sl.dIdx, &sl.idxBytes, b0, cnt, &dI);
      if (r) return r;
      CK(cudaEventRecord(sl.ev[0], ctx->stream));
      r = make_labels_launch(ctx, P, seed, (uint32_t)(perm_first + b0), cnt, dI, (int16_t*)sl.dX, xs);
      if (r) return r;
      CK(cudaEventRecord(sl.ev[1], ctx->stream));
      sl.b0 = b0;
      sl.cnt = cnt;
      return DTO_OK;
    };
    for (long long it = 0; it < std::min<long long>(npipe, 2); ++it) {
      rc = draw(it);
      if (rc) return rc;
      drawn[it] = true;
    }
    // the first batch's results set the ladder
    CK(cudaEventSynchronize(ctx->evSide));
    {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ctx->evk[0], ctx->evk[1]) == cudaSuccess) ctx->acc_perm_ms += ms;
      if (cudaEventElapsedTime(&ms, ctx->evk[2], ctx->evk[3]) == cudaSuccess) ctx->acc_grid_ms += ms;
    }
    unperm = hRes[0];
    take(hRes + 1, 0, cnt0);
    std::vector<double> v(minp.begin(), minp.begin() + cnt0);
    std::sort(v.begin(), v.end());
    const double p90 = std::max(v[(size_t)(kLevel0Quantile * (double)(v.size() - 1))], 1e-300);
    const double p99 = std::max(v[(size_t)(0.99 * (double)(v.size() - 1))], 1e-300);
    const double pmax = std::max(v.back(), 1e-300);
    const int sc = P->fshift;
    const int t0 = fixed_log(p90, sc);
    const int t1 = std::max(fixed_log(p99, sc), t0 + 1);
    const int t2 = std::max((int)std::min(0.0, std::floor((std::log(pmax) + 1.0) * std::ldexp(1.0, sc))), t1 + 1);
    rc = ensure_table(ctx, P, 0, t0);
    if (rc) return rc;
    rc = ensure_table(ctx, P, 1, t1);
    if (rc) return rc;
    rc = ensure_table(ctx, P, 2, t2);
    if (rc) return rc;
    const int nlev = 3;
    // Two batches in flight: while batch b's later table levels, exhaustive
    // fallback and result copy run on the side stream, batch b+1's labels and
    // level-0 table sweep run on the main stream.
    auto harvest = [&](BatchSlot& sl) -> int {
      CK(cudaEventSynchronize(sl.ev[7]));
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, sl.ev[0], sl.ev[1]) == cudaSuccess) ctx->acc_perm_ms += ms;
      if (cudaEventElapsedTime(&ms, sl.ev[2], sl.ev[6]) == cudaSuccess) ctx->acc_grid_ms += ms;
      if (cudaEventElapsedTime(&ms, sl.ev[4], sl.ev[5]) == cudaSuccess) ctx->acc_grid_ms += ms;
      take((const TaskResult*)sl.hRes, sl.b0, sl.cnt);
      ctx->acc_d2h += (long long)sl.cnt * (long long)sizeof(TaskResult);
      sl.busy = false;
      return DTO_OK;
    };
    for (long long it = 0; it < npipe; ++it) {
      BatchSlot& sl = ctx->slot[it & 1];
      if (sl.busy) {
        rc = harvest(sl);
        if (rc) return rc;
      }
      if (!(it < 2 && drawn[it])) {
        rc = draw(it);
        if (rc) return rc;
      }
      const int cnt = sl.cnt;
      int16_t* X = (int16_t*)sl.dX;
      TaskResult* dR = (TaskResult*)sl.dRes;
      CK(cudaEventRecord(sl.ev[2], ctx->stream));
      rc = table_levels(ctx, P, X, xs, cnt, dR, 0, 1, (int*)sl.dFall, sl.dCnt, ctx->stream, 0);
      if (rc) return rc;
      CK(cudaEventRecord(sl.ev[6], ctx->stream));
      CK(cudaStreamWaitEvent(ctx->side, sl.ev[6], 0));
      CK(cudaEventRecord(sl.ev[4], ctx->side));
      rc = table_levels(ctx, P, X, xs, cnt, dR, 1, nlev, (int*)sl.dFall, sl.dCnt, ctx->side, 1);
      if (rc) return rc;
      rc = table_exhaustive(ctx, P, X, xs, cnt, dR, nlev, (const int*)sl.dFall, sl.dCnt, ctx->side);
      if (rc) return rc;
      CK(cudaEventRecord(sl.ev[5], ctx->side));
      CK(cudaMemcpyAsync(sl.hRes, dR, (size_t)cnt * sizeof(TaskResult), cudaMemcpyDeviceToHost, ctx->side));
      CK(cudaEventRecord(sl.ev[7], ctx->side));
      sl.busy = true;
    }
    for (BatchSlot& sl : ctx->slot) {
      if (sl.busy) {
        rc = harvest(sl);
        if (rc) return rc;
      }
    }
    // the main stream's timing event follows the side stream's last work
    CK(cudaEventRecord(ctx->evSide, ctx->side));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->evSide, 0));
  }
  fill_result(P, unperm, 0, out_unpermuted);
  const double p_obs = unperm.p;
  long long count_le = 0;
  for (long long q = 0; q < n_perm; ++q) count_le += (minp[(size_t)q] <= p_obs);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  unsigned long long refined[3] = {0, 0, 0};
  CK(cudaMemcpyAsync(refined, ctx->dRefined, sizeof(refined), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (out_summary) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    dto_summary& s = *out_summary;
    s.n_perm = n_perm;
    s.count_le = count_le;
    s.empirical_pvalue = n_perm > 0 ? (double)count_le / (double)n_perm : 1.0;
    s.fdr = dto_fdr(out_unpermuted->set1_len, out_unpermuted->set2_len, out_unpermuted->intersection_size,
                    P->npop, 0.8);
    s.logp_err_bound_screen = precision == DTO_PRECISION_SCREEN ? 4.5 * std::ldexp(1.0, -P->fshift) : 0.0;
    s.logp_err_bound_fp64 = 2.0e-13;
    s.n_fallback = (int64_t)refined[2];
    s.n_refined = (int64_t)refined[0];
    s.n_stage2 = (int64_t)refined[1];
    s.device_ms = ms;
    s.grid_ms = ctx->acc_grid_ms;
    s.perm_ms = ctx->acc_perm_ms;
    s.n_launches = ctx->acc_launches;
    s.h2d_bytes = ctx->acc_h2d;
    s.d2h_bytes = ctx->acc_d2h + 16;
  }
  return DTO_OK;
}

int dto_optimize(dto_ctx* ctx, dto_pair* P, int permute, uint64_t seed, uint32_t perm_id, const int32_t* idx1,
                 const int32_t* idx2, int precision, dto_result* out) {
  if (!ctx || !P || P->ctx != ctx || !out) return set_err(ctx, DTO_ERR_INVALID, "null argument");
  if (precision != DTO_PRECISION_FP64 && precision != DTO_PRECISION_SCREEN)
    return set_err(ctx, DTO_ERR_INVALID, "unknown precision");
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  const int mode = precision == DTO_PRECISION_FP64 ? kModeFull64 : kModeScreen;
  int rc = grow(ctx, &ctx->dRes, &ctx->resBytes, 2 * sizeof(TaskResult));
  if (rc) return rc;
  rc = grow_host(ctx, &ctx->hRes, &ctx->hResBytes, 2 * sizeof(TaskResult));
  if (rc) return rc;
  const int16_t* dX = P->dYlab;
  void* dIdx = nullptr;
  struct Guard { void*& p; ~Guard() { if (p) cudaFree(p); } } guard{dIdx};
  if (permute) {
    const int32_t* dI = nullptr;
    if (idx1 && idx2) {
      if (!check_perm(idx1, P->N1) || !check_perm(idx2, P->N2))
        return set_err(ctx, DTO_ERR_INVALID, "index array is not a permutation");
      CK(cudaMalloc(&dIdx, (size_t)(P->N1 + P->N2) * 4));
      CK(cudaMemcpyAsync(dIdx, idx1, (size_t)P->N1 * 4, cudaMemcpyHostToDevice, ctx->stream));
      CK(cudaMemcpyAsync((int32_t*)dIdx + P->N1, idx2, (size_t)P->N2 * 4, cudaMemcpyHostToDevice, ctx->stream));
      dI = (const int32_t*)dIdx;
    }
    rc = make_labels(ctx, P, seed, perm_id, 1, dI);
    if (rc) return rc;
    dX = (const int16_t*)ctx->dX;
  }
  rc = grid_tasks(ctx, P, dX, xstride_of(P->N1), 1, mode, (TaskResult*)ctx->dRes);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->hRes, ctx->dRes, sizeof(TaskResult), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  fill_result(P, ((TaskResult*)ctx->hRes)[0], permute ? 1 : 0, out);
  return DTO_OK;
}

int dto_grid_dump(dto_ctx* ctx, dto_pair* P, const int32_t* idx1, const int32_t* idx2, dto_result* records) {
  if (!ctx || !P || P->ctx != ctx || !records) return set_err(ctx, DTO_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  const long long ncell = (long long)P->T1.size() * (long long)P->T2.size();
  int rc = grow(ctx, &ctx->dRes, &ctx->resBytes, 2 * sizeof(TaskResult));
  if (rc) return rc;
  void* dK = nullptr;
  void* dP = nullptr;
  void* dIdx = nullptr;
  struct Guard3 { void*& a; void*& b; void*& c; ~Guard3() { if (a) cudaFree(a); if (b) cudaFree(b); if (c) cudaFree(c); } } guard{dK, dP, dIdx};
  CK(cudaMalloc(&dK, (size_t)ncell * 4));
  CK(cudaMalloc(&dP, (size_t)ncell * 8));
  const int16_t* dX = P->dYlab;
  if (idx1 && idx2) {
    if (!check_perm(idx1, P->N1) || !check_perm(idx2, P->N2))
      return set_err(ctx, DTO_ERR_INVALID, "index array is not a permutation");
    CK(cudaMalloc(&dIdx, (size_t)(P->N1 + P->N2) * 4));
    CK(cudaMemcpyAsync(dIdx, idx1, (size_t)P->N1 * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync((int32_t*)dIdx + P->N1, idx2, (size_t)P->N2 * 4, cudaMemcpyHostToDevice, ctx->stream));
    rc = make_labels(ctx, P, 0, 0, 1, (const int32_t*)dIdx);
    if (rc) return rc;
    dX = (const int16_t*)ctx->dX;
  }
  rc = grid_tasks(ctx, P, dX, xstride_of(P->N1), 1, kModeDump, (TaskResult*)ctx->dRes, (int*)dK, (double*)dP);
  if (rc) return rc;
  std::vector<int> hk((size_t)ncell);
  std::vector<double> hp((size_t)ncell);
  CK(cudaMemcpyAsync(hk.data(), dK, (size_t)ncell * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(hp.data(), dP, (size_t)ncell * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const int permuted = (idx1 && idx2) ? 1 : 0;
  const long long nt2 = (long long)P->T2.size();
  for (long long c = 0; c < ncell; ++c) {
    TaskResult r{hp[(size_t)c], (int)(c / nt2), (int)(c % nt2), hk[(size_t)c], 0};
    fill_result(P, r, permuted, &records[c]);
  }
  return DTO_OK;
}

int dto_hypergeom_sf(dto_ctx* ctx, const int64_t* N, const int64_t* K, const int64_t* n, const int64_t* k,
                     double* out, int64_t count) {
  if (!ctx || count < 0 || (count > 0 && (!N || !K || !n || !k || !out))) return set_err(ctx, DTO_ERR_INVALID, "null argument");
  if (count == 0) return DTO_OK;
  std::lock_guard<std::mutex> g(ctx->mu);
  long long nmax = 0;
  std::vector<long long> q((size_t)count * 4);
  for (int64_t t = 0; t < count; ++t) {
    if (N[t] < 0 || K[t] < 0 || n[t] < 0 || k[t] < 0 || K[t] > N[t] || n[t] > N[t] || N[t] > 4000000)
      return set_err(ctx, DTO_ERR_INVALID, "Failed to create hypergeometric distribution");
    nmax = std::max<long long>(nmax, N[t]);
    q[(size_t)t * 4] = N[t];
    q[(size_t)t * 4 + 1] = K[t];
    q[(size_t)t * 4 + 2] = n[t];
    q[(size_t)t * 4 + 3] = k[t];
  }
  CK(cudaSetDevice(ctx->device));
  int rc = ensure_lf(ctx, nmax);
  if (rc) return rc;
  void* dq = nullptr;
  void* dout = nullptr;
  struct Guard2 { void*& a; void*& b; ~Guard2() { if (a) cudaFree(a); if (b) cudaFree(b); } } guard{dq, dout};
  CK(cudaMalloc(&dq, q.size() * 8));
  CK(cudaMalloc(&dout, (size_t)count * 8));
  CK(cudaMemcpyAsync(dq, q.data(), q.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_sf_batch(ctx->dLF, (const long long*)dq, (double*)dout, count, ctx->stream));
  CK(cudaMemcpyAsync(out, dout, (size_t)count * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return DTO_OK;
}

int dto_export_permutations(dto_ctx* ctx, dto_pair* P, uint64_t seed, uint32_t perm_first, int64_t count,
                            int32_t* idx1, int32_t* idx2) {
  if (!ctx || !P || P->ctx != ctx || count < 0 || (count > 0 && (!idx1 || !idx2)))
    return set_err(ctx, DTO_ERR_INVALID, "null argument");
  if (count == 0) return DTO_OK;
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  int rc = grow(ctx, &ctx->dSig, &ctx->sigBytes, (size_t)count * (P->N1 + P->N2) * 4);
  if (rc) return rc;
  int* sig = (int*)ctx->dSig;
  PermArgs a{};
  a.seed = seed;
  a.pair_id = P->pair_id;
  a.perm_base = perm_first;
  a.L = (int)P->N1;
  a.list_tag = 1;
  a.sigma = sig;
  a.sstride = P->N1;
  CK(launch_perm(a, (int)count, ctx->stream));
  if (!P->same_set) {
    a.L = (int)P->N2;
    a.list_tag = 2;
    a.sigma = sig + count * P->N1;
    a.sstride = P->N2;
    CK(launch_perm(a, (int)count, ctx->stream));
  }
  CK(cudaMemcpyAsync(idx1, sig, (size_t)count * P->N1 * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (!P->same_set)
    CK(cudaMemcpyAsync(idx2, sig + count * P->N1, (size_t)count * P->N2 * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (P->same_set)
    for (int64_t b = 0; b < count; ++b)
      for (int64_t p = 0; p < P->N2; ++p) idx2[b * P->N2 + p] = (int32_t)p;
  return DTO_OK;
}

int dto_run_range_noalloc(dto_ctx* ctx, dto_pair* P, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                          double* d_minp) {
  if (!ctx || !P || P->ctx != ctx || n_perm < 0 || (n_perm > 0 && !d_minp))
    return set_err(ctx, DTO_ERR_INVALID, "dto_run_range_noalloc: null argument");
  if ((long long)perm_first + n_perm > 0xffffffffLL)
    return set_err(ctx, DTO_ERR_INVALID, "dto_run_range_noalloc: permutation ids out of range");
  std::lock_guard<std::mutex> g(ctx->mu);
  CK(cudaSetDevice(ctx->device));
  void* base = nullptr;
  size_t cap = 0;
  CK(noalloc_scratch(ctx->device, &base, &cap));
  if (n_perm == 0) return DTO_OK;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const long long xs = xstride_of(P->N1);
  const size_t per_perm = sizeof(TaskResult) + (size_t)xs * 2 + (P->same_set ? 0 : (size_t)(P->N1 + P->N2) * 4);
  const size_t off_res = 256;
  const size_t off_x = off_res + al((size_t)n_perm * sizeof(TaskResult));
  const size_t off_sig = off_x + al((size_t)n_perm * xs * 2);
  const size_t end = off_sig + (P->same_set ? 0 : al((size_t)n_perm * (P->N1 + P->N2) * 4));
  if (end > cap) {
    const long long most = (long long)((cap - 256 - 3 * 256) / per_perm);
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "dto_run_range_noalloc: n_perm %lld exceeds the %zu-byte device scratch; at most %lld "
                  "permutations of this pair per call",
                  (long long)n_perm, cap, most);
    return set_err(ctx, DTO_ERR_INVALID, msg);
  }
  unsigned char* b8 = (unsigned char*)base;
  int* work = (int*)b8;
  TaskResult* res = (TaskResult*)(b8 + off_res);
  int16_t* X = (int16_t*)(b8 + off_x);
  int* sig = (int*)(b8 + off_sig);
  const int cnt = (int)n_perm;
  PermArgs a{};
  a.seed = seed;
  a.pair_id = P->pair_id;
  a.perm_base = perm_first;
  a.xstride = xs;
  if (P->same_set) {
    a.L = (int)P->N1;
    a.list_tag = 1;
    a.Ylab = P->dYlab;
    a.X = X;
    CK(launch_perm(a, cnt, ctx->stream));
  } else {
    const long long ss = P->N1 + P->N2;
    a.L = (int)P->N1;
    a.list_tag = 1;
    a.sigma = sig;
    a.sstride = ss;
    CK(launch_perm(a, cnt, ctx->stream));
    a.L = (int)P->N2;
    a.list_tag = 2;
    a.sigma = sig + P->N1;
    CK(launch_perm(a, cnt, ctx->stream));
    ComposeArgs c{};
    c.N1 = (int)P->N1;
    c.N2 = (int)P->N2;
    c.idx1 = sig;
    c.idx2 = sig + P->N1;
    c.stride = ss;
    c.map12 = P->dMap12;
    c.lab2 = P->dLab2;
    c.X = X;
    c.xstride = xs;
    CK(launch_compose(c, cnt, ctx->stream));
  }
  CK(cudaMemsetAsync(work, 0, 256, ctx->stream));  // the shared task counter starts at zero
  GridArgs gk{};
  gk.P = P->dev;
  gk.P.LF = ctx->dLF;
  gk.X = X;
  gk.xstride = xs;
  gk.ntask = cnt;
  gk.mode = kModeScreen;
  gk.smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1) <= ctx->smem_optin ? 1 : 0;
  gk.out = res;
  gk.work = work;
  const int ctas = std::max(1, std::min(ctx->nsm, (cnt + kGridWarps - 1) / kGridWarps));
  CK(launch_grid(gk, ctas, ctx->stream));
  CK(launch_noalloc_copy_p(res, d_minp, cnt, ctx->stream));
  return DTO_OK;
}

}  // extern "C"
