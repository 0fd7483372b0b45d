// dto_lane.cpp -- the permutation-null driver: one run of dto_run_range on
// one lane (streams, events, scratch and table screens of its own).
//
// A run replaces run_single_node (src/run/single_node.rs:83-137) over the
// tasks of src/main.rs:122-126: task 0 is the unpermuted pair, tasks 1..P the
// permutations, each reduced to its minimum p (src/dto/optimize_main.rs:53-118),
// and the empirical p-value is #{perm p <= observed p} / P
// (src/stat_operations/empirical_pvalue.rs:109-187).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dto_host.h"

namespace dto {

// Quantile of a sample of minimum p-values (a run's first batch, or the
// pair's previous run) that sets the level-0 table.  With the later levels
// cascaded in the same sweep, 100,000 permutations measured (N = 20,000 /
// 6,000): 0.75 -> 24.2 / 14.4 ms, 0.80 -> 23.8 / 14.2, 0.85 -> 23.7 / 14.5,
// 0.90 -> 23.9 / 15.3, 0.95 -> 26.8 / 18.1.
constexpr double kLevel0Quantile = 0.85;
const double kLevel0QuantileDefault = kLevel0Quantile;
// Permutations of the first batch, whose minimum p-values set the ladder
// (cold runs at 100,000 permutations, N = 20,000: 256 -> 47.8 ms, 512 -> 46.9,
// 1,024 -> 49.3; its slowest tasks and its size both delay the pipeline).
constexpr long long kFirstBatch = 512;
constexpr long long kShortTableMin = 256;  // shortest screen run that takes or leaves a ladder
// Levels of the table ladder: the level-0 quantile, the 99th percentile and
// the maximum + 1 nat (a two-level ladder measured much slower).
constexpr int kLadderLevels = 3;
// Tighter tables a sweep may switch to, for the levels below kTightLevels.
constexpr int kTightTables = 3;
static_assert(kTightTables >= 0 && kTightTables <= 3, "at most three tighter tables");
constexpr int kTightLevels = 3;
// The first batch's screen with a CTA per task (see grid_kernel).
constexpr bool kFirstBatchCoop = true;
// How far (in nats of ln p) a run's ladder bound may lie from the pair's
// stored one before it replaces it.
constexpr double kLadderSlack = 0.25;
// Runs shorter than this build no tighter tables: a short run (most pairs of
// a batch, most served requests) does not repay their builds (the 512-pair
// batch of 10,000 permutations each: 3.00 M perms/s with level 0's three,
// 3.12 M without).
constexpr long long kTightAllMin = 32768;

int set_err(dto_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_err(dto_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_err(ctx, e == cudaErrorMemoryAllocation ? DTO_ERR_OOM : DTO_ERR_CUDA, m);
}

int lane_err(Lane* L, int code, const std::string& msg) {
  if (L && L->err) *L->err = msg;
  return code;
}

int lane_cuda_err(Lane* L, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return lane_err(L, e == cudaErrorMemoryAllocation ? DTO_ERR_OOM : DTO_ERR_CUDA, m);
}

int lane_grow(Lane* L, void** p, size_t* cap, size_t need) {
  if (need <= *cap) return DTO_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t sz = std::max(need, (size_t)4096);
  LCK(cudaMalloc(p, sz));
  *cap = sz;
  return DTO_OK;
}

int lane_grow_host(Lane* L, void** p, size_t* cap, size_t need) {
  if (need <= *cap) return DTO_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  size_t sz = std::max(need, (size_t)4096);
  LCK(cudaMallocHost(p, sz));
  *cap = sz;
  return DTO_OK;
}

int lane_create(dto_ctx* ctx, Lane** out, std::string* err_sink) {
  *out = nullptr;
  Lane* L = new Lane();
  L->ctx = ctx;
  L->err = err_sink ? err_sink : &L->own_err;
  auto fail = [&](cudaError_t e, const char* what) {
    const int rc = lane_cuda_err(L, e, what);
    if (!err_sink && ctx) ctx->err = L->own_err;
    lane_destroy(L);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
  // The side stream runs a run's first batch or unpermuted task and each
  // batch's fallbacks while the main stream sweeps the next batch, at the
  // lowest priority: the highest, which lets its CTAs go first whenever SMs
  // free up, measured neutral at N = 20,000.
  int prio_least = 0, prio_greatest = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest)) != cudaSuccess) return fail(e, "stream");
  if ((e = cudaStreamCreateWithPriority(&L->side, cudaStreamNonBlocking, prio_least)) !=
      cudaSuccess)
    return fail(e, "stream");
  // the table stream builds a run's table screens while its labels are
  // drawn, at the highest priority: its blocks take SM room first as
  // permutation CTAs retire
  if ((e = cudaStreamCreateWithPriority(&L->tstream, cudaStreamNonBlocking, prio_greatest)) != cudaSuccess)
    return fail(e, "stream");
  if ((e = cudaEventCreateWithFlags(&L->evTab, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
  if ((e = cudaEventCreateWithFlags(&L->evSide, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
  if ((e = cudaEventCreate(&L->ev0)) != cudaSuccess) return fail(e, "event");
  if ((e = cudaEventCreate(&L->ev1)) != cudaSuccess) return fail(e, "event");
  for (int q = 0; q < 4; ++q)
    if ((e = cudaEventCreate(&L->evk[q])) != cudaSuccess) return fail(e, "event");
  if ((e = cudaMalloc(&L->dWork, 256)) != cudaSuccess) return fail(e, "scratch");
  if ((e = cudaMalloc(&L->dRefined, 256)) != cudaSuccess) return fail(e, "scratch");
  if ((e = cudaMalloc(&L->dGuess, 2048)) != cudaSuccess) return fail(e, "scratch");
  *out = L;
  return DTO_OK;
}

void lane_destroy(Lane* L) {
  if (!L) return;
  if (L->stream) cudaStreamSynchronize(L->stream);
  if (L->side) cudaStreamSynchronize(L->side);
  if (L->tstream) cudaStreamSynchronize(L->tstream);
  cudaFree(L->dX);
  for (Lane::WaveBuf& wb : L->wave) {
    cudaFree(wb.dX);
    cudaFree(wb.dRes);
    cudaFreeHost(wb.hRes);
    cudaFree(wb.dAux);
    cudaFree(wb.dSegs);
    cudaFreeHost(wb.hSegs);
    for (cudaEvent_t e : wb.ev)
      if (e) cudaEventDestroy(e);
  }
  cudaFree(L->dSig);
  cudaFree(L->dRes);
  cudaFreeHost(L->hRes);
  cudaFree(L->dWork);
  cudaFree(L->dRefined);
  cudaFree(L->dGuess);
  for (void* h : L->dHits) cudaFree(h);
  for (int l = 0; l < Lane::kTables; ++l) cudaFree(L->dKthr[l]);
  for (BatchSlot& sl : L->slot) {
    if (sl.side) {
      cudaStreamSynchronize(sl.side);
      cudaStreamDestroy(sl.side);
    }
    cudaFree(sl.dX);
    cudaFree(sl.dRes);
    cudaFreeHost(sl.hRes);
    cudaFree(sl.dFall);
    cudaFree(sl.dIdx);
    cudaFree(sl.dCnt);
    for (cudaEvent_t e : sl.ev)
      if (e) cudaEventDestroy(e);
  }
  if (L->ev0) cudaEventDestroy(L->ev0);
  if (L->ev1) cudaEventDestroy(L->ev1);
  for (int q = 0; q < 4; ++q)
    if (L->evk[q]) cudaEventDestroy(L->evk[q]);
  if (L->evSide) cudaEventDestroy(L->evSide);
  if (L->evTab) cudaEventDestroy(L->evTab);
  if (L->tstream) cudaStreamDestroy(L->tstream);
  if (L->side) cudaStreamDestroy(L->side);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
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
  o->status = DTO_OK;
  o->route = r.route;
  o->reserved = 0;
}

// Batch size of a run: 2^32 bytes of labels (4 GiB), and at
// most 1 GiB of index scratch for test mode and for pairs whose lists hold
// different features.  Every launch pays a tail (its slowest tasks), so
// fewer, larger batches win: per 100,000 permutations at N = 20,000, 4 GiB
// (one batch) measured 22.6 ms against 23.8 ms for 2 GiB (two); before the
// cascade 2 GiB measured 36.2 ms at N = 20,000 and 39.6 ms on the
// 18,000-feature background pair, 1 GiB 36.2-36.8 and 43.1 ms, 512 MiB
// 40-41 ms and 46 ms.

long long batch_of(const dto_pair* P, int64_t n_perm, bool test_mode) {
  const long long xs = xstride_of(P->N1);
  const long long L12 = P->N1 + P->N2;
  long long batch = std::max(1LL, std::min<long long>((1LL << 32) / (xs * 2), 1LL << 20));
  if (test_mode || !P->same_set) batch = std::min(batch, std::max(1LL, (1LL << 30) / (L12 * 4)));
  return std::min<long long>(batch, std::max<long long>(n_perm, 1));
}

long long run_device_bytes(const dto_ctx* ctx, const dto_pair* P, int64_t n_perm, bool test_mode) {
  const long long xs = xstride_of(P->N1);
  const long long L12 = P->N1 + P->N2;
  const long long batch = batch_of(P, n_perm, test_mode);
  const long long first = std::min<long long>(batch, 1025);
  long long b = first * xs * 2 + (long long)(batch + 1) * (long long)sizeof(TaskResult);  // first batch
  if (n_perm > 2048) {
    b += Lane::kSlots * batch * (xs * 2 + (long long)sizeof(TaskResult) + 12);                // batch slots
    b += (long long)kTableCtasPerSm * ctx->nsm * kTableWarps * kTableWarpHits * 8;  // hits
    b += (long long)Lane::kTables * (long long)table_entries(P->C, P->dev.n1) * 2;  // tables
  }
  if (test_mode || !P->same_set) b += 2 * batch * L12 * 4;  // index scratch
  return b;
}

int lane_grid_tasks(Lane* L, dto_pair* P, const int16_t* dX, long long xstride, int ntask, int mode,
                    TaskResult* dOut, int* dumpK, double* dumpP, bool guess, cudaStream_t stream, bool coop) {
  if (!stream) stream = L->stream;
  GridArgs a{};
  a.P = P->dev;
  a.P.LF = L->ctx->dLF.load();  // the context's table may have grown since the pair was created
  a.X = dX;
  a.xstride = xstride;
  a.ntask = ntask;
  a.mode = mode;
  a.route = mode == kModeFull64 ? DTO_ROUTE_FP64 : DTO_ROUTE_SCREEN;
  size_t smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1);
  a.smemF = smemF <= L->ctx->smem_optin ? 1 : 0;
  a.out = dOut;
  a.work = L->dWork;
  a.n_refined = L->dRefined;
  a.guess_hist = (guess && mode == kModeScreen) ? L->dGuess : nullptr;
  a.dump_k = dumpK;
  a.dump_p = dumpP;
  a.coop = (coop && mode == kModeScreen) ? 1 : 0;
  LCK(cudaMemsetAsync(L->dWork, 0, sizeof(int), stream));
  int ctas = std::min(L->ctx->nsm, a.coop ? ntask : (ntask + kGridWarps - 1) / kGridWarps);
  ctas = std::max(ctas, 1);
  LCK(cudaEventRecord(L->evk[2], stream));
  LCK(launch_grid(a, ctas, stream));
  LCK(cudaEventRecord(L->evk[3], stream));
  L->acc_launches += 1;
  return DTO_OK;
}

// Table screen `level` for bound tau (fixed-point ln p), built on the device
// into the lane's buffer (kept while the lane runs the same pair and bound).
int ensure_table(Lane* L, dto_pair* P, int level, int tau, cudaStream_t stream, bool* built) {
  if (L->kthr_pair[level] == P->serial && L->kthr_tau[level] == tau) return DTO_OK;
  *built = true;
  int rc = lane_grow(L, (void**)&L->dKthr[level], &L->kthrBytes[level], table_entries(P->C, P->dev.n1) * 2);
  if (rc) return rc;
  TableArgs t{};
  t.n1 = P->dev.n1;
  t.n2 = P->dev.n2;
  t.N = (int)P->npop;
  t.C = 2 * P->C;  // the half-warp sweep reads 16 lanes of 2 C columns
  t.rowstart = P->dRow;
  t.ncnt = P->dNcnt;
  t.F = P->dF;
  t.fshift = P->fshift;
  t.tau = tau;
  t.mcnt = P->dMcnt;
  t.N1 = (int)P->N1;
  t.kthr = L->dKthr[level];
  LCK(launch_table_build(t, L->ctx->nsm, stream));
  L->acc_launches += 1;
  L->kthr_pair[level] = P->serial;
  L->kthr_tau[level] = tau;
  return DTO_OK;
}

// The table ladder over tasks [0, ntask) of X, on `stream` with hit buffer
// `hb`, in one launch: a task with no hit at level l (its minimum lies above
// the level's bound) is swept at level l + 1 by the same half-warp, and the
// last level's misses go to the exhaustive screen's list (table_exhaustive).
// The list and the counts stay on the device: `fall` holds one list of ntask
// entries per level (the last one used), `cnts` 8 task counters then 4 list
// counts (zeroed here).  Levels below `tight_levels` switch to their tighter
// tables.
int table_levels(Lane* L, dto_pair* P, const int16_t* X, long long xstride, int ntask, TaskResult* dOut, int* fall,
                 int* cnts, cudaStream_t stream, int hb, int tight_levels) {
  NvtxRange range("dto: table sweep");
  const int cap = std::max(ntask, 1);
  const int hitcap = kTableWarpHits;
  const int nlev = kLadderLevels;
  int rc = lane_grow(L, &L->dHits[hb], &L->hitBytes[hb], (size_t)kTableCtasPerSm * L->ctx->nsm * kTableWarps * hitcap * 8);
  if (rc) return rc;
  LCK(cudaMemsetAsync(cnts, 0, 12 * sizeof(int), stream));
  TableGridArgs a{};
  a.P = P->dev;
  a.P.LF = L->ctx->dLF.load();
  a.X = X;
  a.xstride = xstride;
  a.ntask = ntask;
  a.tau = L->kthr_tau[0];
  a.kthr = L->dKthr[0];
  a.ntight = 0 < tight_levels ? kTightTables : 0;
  for (int q = 0; q < a.ntight; ++q) {
    a.tight[q] = L->dKthr[tight_slot(0, q)];
    a.tight_tau[q] = L->kthr_tau[tight_slot(0, q)];
  }
  a.nlev = nlev;
  for (int l = 1; l < nlev; ++l) {
    a.kthr_up[l - 1] = L->dKthr[l];
    a.tau_up[l - 1] = L->kthr_tau[l];
    a.ntight_up[l - 1] = l < tight_levels ? kTightTables : 0;
    for (int q = 0; q < a.ntight_up[l - 1]; ++q) {
      a.tight_up[l - 1][q] = L->dKthr[tight_slot(l, q)];
      a.tight_tau_up[l - 1][q] = L->kthr_tau[tight_slot(l, q)];
    }
  }
  a.route = DTO_ROUTE_LEVEL0;
  a.smemF = table_smem_bytes(P->C, P->dev.n1, P->dev.n2, P->npop, 1) <= L->ctx->smem_optin ? 1 : 0;
  a.out = dOut;
  a.work = cnts;
  a.n_refined = L->dRefined;
  a.fallback = fall + (size_t)(nlev - 1) * cap;
  a.nfallback = cnts + 8 + nlev - 1;
  a.hitbuf = (int2*)L->dHits[hb];
  a.hitcap = hitcap;
  const int ctas = std::max(1, std::min(kTableCtasPerSm * L->ctx->nsm, ntask / (kTableWarps * 2) + 1));
  LCK(launch_table_grid(a, P->C, ctas, stream));
  L->acc_launches += 1;
  return DTO_OK;
}

// The exhaustive screen of what the last table level left, on `stream`.
int table_exhaustive(Lane* L, dto_pair* P, const int16_t* X, long long xstride, int ntask, TaskResult* dOut,
                     int nlev, const int* fall, int* cnts, cudaStream_t stream, unsigned long long* refined) {
  NvtxRange range("dto: exhaustive fallback");
  const int cap = std::max(ntask, 1);
  GridArgs g{};
  g.P = P->dev;
  g.P.LF = L->ctx->dLF.load();
  g.X = X;
  g.xstride = xstride;
  g.ntask = ntask;
  g.mode = kModeScreen;
  g.route = DTO_ROUTE_FALLBACK;
  g.hwlab = 1;  // a table run's labels
  g.smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1) <= L->ctx->smem_optin ? 1 : 0;
  g.coop = 1;  // the few tasks left here are the hard ones: a CTA each
  g.out = dOut;
  g.work = cnts + nlev;
  g.n_refined = refined ? refined : L->dRefined;
  g.task_list = fall + (size_t)(nlev - 1) * cap;
  g.ntask_dev = cnts + 8 + nlev - 1;
  LCK(launch_grid(g, L->ctx->nsm, stream));
  L->acc_launches += 1;
  return DTO_OK;
}

void LadderModel::record(const LadderShape& x) {
  std::lock_guard<std::mutex> g(mu);
  for (auto it = shapes.begin(); it != shapes.end(); ++it)
    if (it->npop == x.npop && it->N1 == x.N1 && it->N2 == x.N2 && it->ncommon == x.ncommon && it->n1 == x.n1 &&
        it->n2 == x.n2 && it->same_set == x.same_set) {
      shapes.erase(it);
      break;
    }
  if (shapes.size() >= kMaxShapes) shapes.erase(shapes.begin());
  shapes.push_back(x);
}

bool LadderModel::fits(const LadderShape& x, const LadderShape& want, double* dist) {
  auto rel = [](double a, double b) { return std::fabs(a - b) / std::max(1.0, std::max(a, b)); };
  if (x.same_set != want.same_set) return false;
  const double d[6] = {rel((double)x.npop, (double)want.npop), rel((double)x.N1, (double)want.N1),
                       rel((double)x.N2, (double)want.N2), rel((double)x.ncommon, (double)want.ncommon),
                       rel(x.n1, want.n1), rel(x.n2, want.n2)};
  double sum = 0.0;
  bool ok = true;
  for (double v : d) {
    ok = ok && v <= kTol;
    sum += v;
  }
  if (dist) *dist = sum;
  return ok;
}

bool LadderModel::lookup(const LadderShape& want, double nats[kLadderTaus], double* q0) {
  std::lock_guard<std::mutex> g(mu);
  const LadderShape* best = nullptr;
  double best_d = 1e300;
  for (const LadderShape& x : shapes) {
    double sum = 0.0;
    if (fits(x, want, &sum) && sum < best_d) {
      best_d = sum;
      best = &x;
    }
  }
  if (!best) return false;
  for (int l = 0; l < kLadderTaus; ++l) nats[l] = best->nats[l];
  if (q0) *q0 = best->q0;
  return true;
}

LadderShape shape_of(const dto_pair* P) {
  LadderShape x{};
  x.npop = P->npop;
  x.N1 = P->N1;
  x.N2 = P->N2;
  x.ncommon = P->ncommon;
  x.n1 = (int)P->T1.size();
  x.n2 = (int)P->T2.size();
  x.same_set = P->same_set;
  return x;
}

int fixed_log(double p, int fshift) {
  double t = std::floor(std::log(p) * std::ldexp(1.0, fshift));
  return (int)std::max(-2.0e9, std::min(0.0, t));
}

// Labels of n_perm permutations starting at perm id `first` into L->dX.
int lane_make_labels(Lane* L, dto_pair* P, uint64_t seed, uint32_t first, int count,
                     const int32_t* dIdx /* nullable: test mode, [count][N1+N2] */, int row0) {
  NvtxRange range("dto: labels");
  long long xs = xstride_of(P->N1);
  int rc = lane_grow(L, &L->dX, &L->xBytes, (size_t)(count + row0) * xs * 2);
  if (rc) return rc;
  int16_t* X = (int16_t*)L->dX + (size_t)row0 * xs;
  LCK(cudaEventRecord(L->evk[0], L->stream));
  rc = make_labels_launch(L, P, seed, first, count, dIdx, X, xs);
  LCK(cudaEventRecord(L->evk[1], L->stream));
  return rc;
}

int make_labels_launch(Lane* L, dto_pair* P, uint64_t seed, uint32_t first, int count,
                       const int32_t* dIdx, int16_t* X, long long xs, bool hwlab) {
  int rc = DTO_OK;
  const int16_t* lab1 = hwlab ? P->dYlabHw : P->dYlab;  // the labels' form (hwlab: a table run's)
  const int16_t* lab2 = hwlab ? P->dLab2Hw : P->dLab2;
  if (dIdx) {
    ComposeArgs c{};
    c.N1 = (int)P->N1;
    c.N2 = (int)P->N2;
    c.idx1 = dIdx;
    c.idx2 = dIdx + P->N1;
    c.stride = P->N1 + P->N2;
    c.map12 = P->dMap12;
    c.lab2 = lab2;
    c.X = X;
    c.xstride = xs;
    LCK(launch_compose(c, count, L->stream));
    L->acc_launches += 1;
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
    a.Ylab = lab1;
    a.X = X;
    a.rowstart = P->dRow;
    a.n1 = P->dev.n1;
    LCK(launch_perm(a, count, L->stream));
    L->acc_launches += 1;
    return DTO_OK;
  }
  long long ss = P->N1 + P->N2;
  rc = lane_grow(L, &L->dSig, &L->sigBytes, (size_t)count * ss * 4);
  if (rc) return rc;
  int* sig = (int*)L->dSig;
  a.L = (int)P->N1;
  a.list_tag = 1;
  a.sigma = sig;
  a.sstride = ss;
  LCK(launch_perm(a, count, L->stream));
  a.L = (int)P->N2;
  a.list_tag = 2;
  a.sigma = sig + P->N1;
  LCK(launch_perm(a, count, L->stream));
  ComposeArgs c{};
  c.N1 = (int)P->N1;
  c.N2 = (int)P->N2;
  c.idx1 = sig;
  c.idx2 = sig + P->N1;
  c.stride = ss;
  c.map12 = P->dMap12;
  c.lab2 = lab2;
  c.X = X;
  c.xstride = xs;
  LCK(launch_compose(c, count, L->stream));
  L->acc_launches += 3;
  return DTO_OK;
}

// Bounds of the table levels from a sample of minimum p-values: the
// kLevel0Quantile quantile (level 0), the 99th percentile (level 1), one nat above the maximum
// (level 2), as fixed-point ln p, each above the one before; then each
// level's three tighter tables (kLadderTaus entries in all).
// The ladder's order: each level's bound above the one before, each level's
// tighter tables below its bound and below one another.
void ladder_order(int tau[kLadderTaus]) {
  tau[1] = std::max(tau[1], tau[0] + 1);
  tau[2] = std::max(tau[2], tau[1] + 1);
  if (kLadderLevels == 2) tau[1] = tau[2];
  for (int l = 0; l < 3; ++l) {
    int prev = tau[l];
    for (int t = 0; t < 3; ++t) {
      tau[tight_slot(l, t)] = std::min(tau[tight_slot(l, t)], prev - 1);
      prev = tau[tight_slot(l, t)];
    }
  }
}

namespace {

// An evenly strided sample of at most 16,384 minima (the permutations are in
// random order).
std::vector<double> ladder_sample_of(const std::vector<double>& all) {
  const size_t stride = std::max<size_t>((all.size() + 16383) / 16384, 1);
  std::vector<double> v;
  v.reserve(all.size() / stride + 1);
  for (size_t i = 0; i < all.size(); i += stride) v.push_back(all[i]);
  return v;
}

// The bounds from a sample (reordered by the selections) and the maximum of
// all the minima.
void ladder_taus(std::vector<double>& v, double pmax_all, int fshift, int tau[kLadderTaus], double q0) {
  auto q = [&](double f) {
    const size_t k = (size_t)(f * (double)(v.size() - 1));
    std::nth_element(v.begin(), v.begin() + (long)k, v.end());
    return std::max(v[k], 1e-300);
  };
  const double p0 = q(q0 > 0.0 ? q0 : kLevel0Quantile);
  const double p99 = q(0.99);
  const double pmax = std::max(pmax_all, 1e-300);
  tau[0] = fixed_log(p0, fshift);
  tau[1] = fixed_log(p99, fshift);
  tau[2] = (int)std::min(0.0, std::floor((std::log(pmax) + 1.0) * std::ldexp(1.0, fshift)));
  // the tighter tables a sweep switches to once a task's bound is known,
  // each below the one before: for level 0 the 60th, 25th and 5th
  // percentiles (100,000 permutations at N = 20,000 / 6,000 and 200,000 of
  // the 18,000-feature background pair: 22.45 / 14.36 / 47.8 ms against
  // 22.54 / 14.50 / 48.5 ms for the 50th, 10th and 1st), for level 1 the
  // 98th, 96th and 93rd, for level 2 the maximum, the 99.9th and the 99.5th
  const double ptight[3][3] = {{q(0.6), q(0.25), q(0.05)}, {q(0.98), q(0.96), q(0.93)}, {pmax, q(0.999), q(0.995)}};
  for (int l = 0; l < 3; ++l)
    for (int t = 0; t < 3; ++t) tau[tight_slot(l, t)] = fixed_log(ptight[l][t], fshift);
  ladder_order(tau);
}

// New bounds t into the pair's ladder (those that moved by more than
// kLadderSlack nats; the bounds are quantiles of the pair's null
// distribution, so another seed moves them a little, and a kept bound spares
// the next run that table's rebuild), and the pair's shape into the
// context's model.  The caller holds P->ladder_mu.
void ladder_apply(dto_ctx* ctx, dto_pair* P, const int t[kLadderTaus], double q0) {
  const long long slack = (long long)std::ldexp(kLadderSlack, P->fshift);
  for (int l = 0; l < kLadderTaus; ++l)
    if (!P->ladder_ok || std::llabs((long long)t[l] - P->ladder_tau[l]) > slack) P->ladder_tau[l] = t[l];
  ladder_order(P->ladder_tau);
  P->ladder_ok = true;
  LadderShape x = shape_of(P);
  for (int l = 0; l < kLadderTaus; ++l) x.nats[l] = std::ldexp((double)P->ladder_tau[l], -P->fshift);
  x.q0 = q0;
  ctx->ladders.record(x);
}

// The context's pending record into its model; its entry returned.  The
// caller holds ctx->defer_mu.
LadderShape record_deferred(dto_ctx* ctx) {
  LadderPending& r = ctx->deferred_rec;
  int t[kLadderTaus];
  ladder_taus(r.sample, r.pmax, r.fshift, t, r.q0);
  LadderShape x = r.shape;
  for (int l = 0; l < kLadderTaus; ++l) x.nats[l] = std::ldexp((double)t[l], -r.fshift);
  x.q0 = r.q0;
  ctx->ladders.record(x);
  ctx->deferred = false;
  return x;
}

}  // namespace

void ladder_of(const std::vector<double>& all, int fshift, int tau[kLadderTaus], double q0) {
  // the quantiles from a sample, the maximum from all of them
  std::vector<double> v = ladder_sample_of(all);
  ladder_taus(v, *std::max_element(all.begin(), all.end()), fshift, tau, q0);
}

void ladder_update(dto_ctx* ctx, dto_pair* P, const std::vector<double>& minp, bool defer) {
  std::vector<double> sample = ladder_sample_of(minp);
  const double pmax = *std::max_element(minp.begin(), minp.end());
  std::lock_guard<std::mutex> g(P->ladder_mu);
  const double q0 = P->q0 > 0.0 ? P->q0 : kLevel0Quantile;
  P->ladder_sample.swap(sample);
  P->ladder_pmax = pmax;
  if (!defer) {
    std::vector<double> v = P->ladder_sample;
    int t[kLadderTaus];
    ladder_taus(v, pmax, P->fshift, t, q0);
    P->ladder_pending = false;
    ladder_apply(ctx, P, t, q0);
    return;
  }
  P->ladder_pending = true;
  ++P->ladder_gen;
  std::lock_guard<std::mutex> d(ctx->defer_mu);
  // another pair's pending record goes to the model now
  if (ctx->deferred && ctx->deferred_rec.serial != P->serial) record_deferred(ctx);
  LadderPending& r = ctx->deferred_rec;
  r.sample = P->ladder_sample;
  r.pmax = pmax;
  r.q0 = q0;
  r.fshift = P->fshift;
  r.shape = shape_of(P);
  r.serial = P->serial;
  r.gen = P->ladder_gen;
  ctx->deferred = true;
}

void ladder_flush(dto_ctx* ctx, dto_pair* P) {
  std::lock_guard<std::mutex> g(P->ladder_mu);
  if (!P->ladder_pending) return;
  std::vector<double> v = P->ladder_sample;
  const double q0 = P->q0 > 0.0 ? P->q0 : kLevel0Quantile;
  int t[kLadderTaus];
  ladder_taus(v, P->ladder_pmax, P->fshift, t, q0);
  P->ladder_pending = false;
  ladder_apply(ctx, P, t, q0);
  // the context's copy of this update is recorded
  std::lock_guard<std::mutex> d(ctx->defer_mu);
  if (ctx->deferred && ctx->deferred_rec.serial == P->serial && ctx->deferred_rec.gen == P->ladder_gen)
    ctx->deferred = false;
}

void ladder_flush_deferred(dto_ctx* ctx) {
  std::lock_guard<std::mutex> d(ctx->defer_mu);
  if (ctx->deferred) record_deferred(ctx);
}

bool ladder_deferred_fits(dto_ctx* ctx, const LadderShape& want) {
  std::lock_guard<std::mutex> d(ctx->defer_mu);
  return ctx->deferred && LadderModel::fits(ctx->deferred_rec.shape, want);
}

bool ladder_take_deferred(dto_ctx* ctx, const LadderShape& want, double nats[kLadderTaus], double* q0) {
  std::lock_guard<std::mutex> d(ctx->defer_mu);
  if (!ctx->deferred || !LadderModel::fits(ctx->deferred_rec.shape, want)) return false;
  const LadderShape x = record_deferred(ctx);
  for (int l = 0; l < kLadderTaus; ++l) nats[l] = x.nats[l];
  *q0 = x.q0;
  return true;
}

int lane_run_range(Lane* L, dto_pair* P, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                   const int32_t* perm_idx, int precision, dto_result* out_unpermuted, double* out_minp,
                   dto_result* out_perm, dto_summary* out_summary) {
  if (!P) return lane_err(L, DTO_ERR_INVALID, "null argument");
  if (P->ctx != L->ctx) return lane_err(L, DTO_ERR_INVALID, "the pair belongs to another context");
  if (n_perm < 0 || n_perm > 0x7fffffffLL || (long long)perm_first + n_perm > 0xffffffffLL)
    return lane_err(L, DTO_ERR_INVALID, "n_perm out of range");
  if (precision != DTO_PRECISION_FP64 && precision != DTO_PRECISION_SCREEN)
    return lane_err(L, DTO_ERR_INVALID, "unknown precision");
  NvtxRange run_range("dto: run");
  LCK(cudaSetDevice(L->ctx->device));
  const long long L12 = P->N1 + P->N2;
  if (perm_idx) {
    for (long long b = 0; b < n_perm; ++b) {
      if (!check_perm(perm_idx + b * L12, P->N1) || !check_perm(perm_idx + b * L12 + P->N1, P->N2))
        return lane_err(L, DTO_ERR_INVALID, "perm_idx row is not a permutation");
    }
  }
  const int mode = precision == DTO_PRECISION_FP64 ? kModeFull64 : kModeScreen;
  // without out_unpermuted the unpermuted task is not run (a replica that
  // takes a range of permutation ids while another computes the observed p)
  const bool want0 = out_unpermuted != nullptr;
  const long long xs = xstride_of(P->N1);
  const long long batch = batch_of(P, n_perm, perm_idx != nullptr);
  int rc = lane_grow(L, &L->dRes, &L->resBytes, (size_t)(batch + 1) * sizeof(TaskResult));
  if (rc) return rc;
  rc = lane_grow_host(L, &L->hRes, &L->hResBytes, (size_t)(batch + 1) * sizeof(TaskResult));
  if (rc) return rc;
  void* dIdx = nullptr;
  size_t idxBytes = 0;
  struct Guard { void*& p; ~Guard() { if (p) cudaFree(p); } } guard{dIdx};
  TaskResult* dRes = (TaskResult*)L->dRes;
  TaskResult* hRes = (TaskResult*)L->hRes;
  L->acc_grid_ms = L->acc_perm_ms = L->acc_sweep0_ms = 0.0;
  L->acc_launches = L->acc_h2d = L->acc_d2h = L->acc_sweep0_launches = L->acc_sweep0_tasks = 0;
  LCK(cudaMemsetAsync(L->dRefined, 0, 3 * sizeof(unsigned long long), L->stream));
  LCK(cudaMemsetAsync(L->dGuess, 0, 2048, L->stream));
  LCK(cudaEventRecord(L->ev0, L->stream));
  // this run's table builds follow whatever earlier calls left on the main
  // stream (a call that returned early may leave a sweep of the lane's
  // tables running), not this run's own work
  LCK(cudaStreamWaitEvent(L->tstream, L->ev0, 0));
  // a server's cancel request, checked between batches: the work in flight
  // drains and the run returns DTO_ERR_CANCELLED
  auto cancelled = [&]() -> int {
    if (!L->cancel || L->cancel->load() == 0) return DTO_OK;
    cudaStreamSynchronize(L->stream);
    cudaStreamSynchronize(L->side);
    for (BatchSlot& sl : L->slot) {
      if (sl.side) cudaStreamSynchronize(sl.side);
      sl.busy = false;
    }
    return lane_err(L, DTO_ERR_CANCELLED, "the request was cancelled");
  };
  // every entry is written before it is read: the lane's buffer is reused
  // (a run as long as the last one clears nothing)
  std::vector<double>& minp = L->minp;
  minp.resize((size_t)n_perm);
  long long nroute[DTO_ROUTES] = {};
  cudaEvent_t last_l0_end = nullptr;  // end of the last table sweep (main stream)
  TaskResult unperm{};
  // Short runs (and FP64 runs) go through the exhaustive screen in batches,
  // the unpermuted task (task 0) in row 0 of the first.  Long runs go through
  // the table ladder (below).
  const long long first_batch = kFirstBatch;
  // a short screen run of a pair with a ladder of its own (left by any
  // earlier run of at least kShortTableMin permutations) goes through the
  // table sweep as well: no first batch to measure
  bool own_ladder = false;
  {
    std::lock_guard<std::mutex> g(P->ladder_mu);
    own_ladder = P->ladder_ok || P->ladder_pending;
  }
  const bool use_table =
      (mode == kModeScreen) && (n_perm > 2 * first_batch || (own_ladder && n_perm >= kShortTableMin));
  // every task's result must name a grid cell: a result that does not is a
  // device-side failure and is reported instead of read
  const int nt1 = (int)P->T1.size(), nt2 = (int)P->T2.size();
  auto valid = [&](const TaskResult& r) { return r.i >= 0 && r.i < nt1 && r.j >= 0 && r.j < nt2; };
  auto take = [&](const TaskResult* hr, long long b0, int cnt) -> int {
    for (int q = 0; q < cnt; ++q) {
      const TaskResult& r = hr[q];
      if (!valid(r)) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "permutation %lld: the search returned no grid cell",
                      (long long)perm_first + b0 + q);
        return lane_err(L, DTO_ERR_CUDA, msg);
      }
      minp[(size_t)(b0 + q)] = r.p;
      ++nroute[(r.route >= 0 && r.route < DTO_ROUTES) ? r.route : DTO_ROUTE_NONE];
      if (out_minp) out_minp[b0 + q] = r.p;
      if (out_perm) fill_result(P, r, 1, &out_perm[b0 + q]);
    }
    return DTO_OK;
  };
  auto upload_idx = [&](void** buf, size_t* cap, long long b0, int cnt, const int32_t** dI) -> int {
    *dI = nullptr;
    if (!perm_idx || cnt <= 0) return DTO_OK;
    const size_t bytes = (size_t)cnt * L12 * 4;
    int r = lane_grow(L, buf, cap, bytes);
    if (r) return r;
    LCK(cudaMemcpyAsync(*buf, perm_idx + b0 * L12, bytes, cudaMemcpyHostToDevice, L->stream));
    L->acc_h2d += (long long)bytes;
    *dI = (const int32_t*)*buf;
    return DTO_OK;
  };
  if (!use_table) {
    for (long long b0 = 0; b0 < std::max<long long>(n_perm, 1); b0 += batch) {
      if ((rc = cancelled())) return rc;
      const int row0 = (b0 == 0 && want0) ? 1 : 0;
      const int cnt = (int)std::max(0LL, std::min(batch, n_perm - b0));
      const int32_t* dI = nullptr;
      rc = upload_idx(&dIdx, &idxBytes, b0, cnt, &dI);
      if (rc) return rc;
      if (cnt > 0) {
        rc = lane_make_labels(L, P, seed, (uint32_t)(perm_first + b0), cnt, dI, row0);
        if (rc) return rc;
      } else {
        rc = lane_grow(L, &L->dX, &L->xBytes, (size_t)xs * 2);
        if (rc) return rc;
      }
      if (row0) LCK(cudaMemcpyAsync(L->dX, P->dYlab, (size_t)P->N1 * 2, cudaMemcpyDeviceToDevice, L->stream));
      const int ntask = cnt + row0;
      if (ntask == 0) continue;
      rc = lane_grid_tasks(L, P, (const int16_t*)L->dX, xs, ntask, mode, dRes, nullptr, nullptr, true);
      if (rc) return rc;
      LCK(cudaMemcpyAsync(hRes, dRes, (size_t)ntask * sizeof(TaskResult), cudaMemcpyDeviceToHost, L->stream));
      L->acc_d2h += (long long)ntask * (long long)sizeof(TaskResult);
      LCK(cudaStreamSynchronize(L->stream));
      float ms = 0.f;
      if (cnt > 0 && cudaEventElapsedTime(&ms, L->evk[0], L->evk[1]) == cudaSuccess) L->acc_perm_ms += ms;
      if (cudaEventElapsedTime(&ms, L->evk[2], L->evk[3]) == cudaSuccess) L->acc_grid_ms += ms;
      if (row0) unperm = hRes[0];
      if (row0 && !valid(hRes[0])) return lane_err(L, DTO_ERR_CUDA, "unpermuted task: the search returned no grid cell");
      rc = take(hRes + row0, b0, cnt);
      if (rc) return rc;
    }
    // the pair's ladder for its later runs
    if (mode == kModeScreen && n_perm >= kShortTableMin) ladder_update(L->ctx, P, minp, L == L->ctx->lane0);
  } else {
    // Slots left busy by a call that returned early hold nothing of this call.
    LCK(cudaStreamSynchronize(L->side));
    for (BatchSlot& sl : L->slot) {
      if (sl.side) LCK(cudaStreamSynchronize(sl.side));
      sl.busy = false;
    }
    // The ladder: from an earlier run of this pair when there was one (task 0
    // then runs alone on the side stream and every permutation goes through
    // the pipeline), else from this run's first batch: task 0 and first_batch
    // permutations through the exhaustive screen on the side stream.  The
    // first batch's slowest tasks (the permutations with the largest minimum
    // p) take several times a typical task; meanwhile the main stream draws
    // the labels of the first two pipelined batches.
    // A ladder left pending by the pair's last run is made into bounds once
    // this run's labels are on their way.
    int tau[kLadderTaus] = {};
    bool warm = false, pending = false;
    {
      std::lock_guard<std::mutex> g(P->ladder_mu);
      if (P->ladder_ok || P->ladder_pending) {
        warm = true;
        pending = P->ladder_pending;
        for (int l = 0; l < kLadderTaus; ++l) tau[l] = P->ladder_tau[l];
      }
    }
    // a pair of the same shape has run: start from its ladder (and its
    // level-0 quantile, unless this pair has one).  When that run's ladder is
    // still pending, its bounds too are computed once the labels are on
    // their way.
    double model_nats[kLadderTaus], model_q0 = 0.0;
    auto from_model = [&]() {
      {
        std::lock_guard<std::mutex> g(P->ladder_mu);
        if (P->q0 <= 0.0) P->q0 = model_q0;
      }
      const double scale = std::ldexp(1.0, P->fshift);
      for (int l = 0; l < kLadderTaus; ++l)
        tau[l] = (int)std::max(-2.0e9, std::min(0.0, std::floor(model_nats[l] * scale)));
      ladder_order(tau);
    };
    bool model_later = false;
    if (!warm && L->use_model) {
      if (ladder_deferred_fits(L->ctx, shape_of(P))) {
        warm = model_later = true;
      } else if (L->ctx->ladders.lookup(shape_of(P), model_nats, &model_q0)) {
        warm = true;
        from_model();
      }
    }
    const int cnt0 = warm ? 0 : (int)first_batch;
    if (warm) {
      rc = lane_grow(L, &L->dX, &L->xBytes, (size_t)xs * 2);
      if (rc) return rc;
    } else {
      const int32_t* dI0 = nullptr;
      rc = upload_idx(&dIdx, &idxBytes, 0, cnt0, &dI0);
      if (rc) return rc;
      rc = lane_make_labels(L, P, seed, perm_first, cnt0, dI0, 1);
      if (rc) return rc;
    }
    LCK(cudaMemcpyAsync(L->dX, P->dYlab, (size_t)P->N1 * 2, cudaMemcpyDeviceToDevice, L->stream));
    LCK(cudaEventRecord(L->evSide, L->stream));
    LCK(cudaStreamWaitEvent(L->side, L->evSide, 0));
    // task 0 sits in row 0 of the first batch; without want0 only rows 1.. run
    const int r0 = want0 ? 0 : 1;
    const bool first_launch = cnt0 + 1 - r0 > 0;
    if (first_launch) {
      rc = lane_grid_tasks(L, P, (const int16_t*)L->dX + (size_t)r0 * xs, xs, cnt0 + 1 - r0, mode, dRes + r0,
                           nullptr, nullptr, !warm, L->side, warm || (kFirstBatchCoop && L->coop_first));
      if (rc) return rc;
      LCK(cudaMemcpyAsync(hRes + r0, dRes + r0, (size_t)(cnt0 + 1 - r0) * sizeof(TaskResult),
                          cudaMemcpyDeviceToHost, L->side));
      L->acc_d2h += (long long)(cnt0 + 1 - r0) * (long long)sizeof(TaskResult);
    }
    LCK(cudaEventRecord(L->evSide, L->side));
    // Labels of the pipelined batches b = 0, 1, ... (permutations
    // cnt0 + b * batch on), slot b % kSlots; the first two are drawn now.
    const long long pipe_from = cnt0;
    const long long npipe = (n_perm - pipe_from + batch - 1) / batch;
    bool drawn[2] = {false, false};
    auto draw = [&](long long it) -> int {
      BatchSlot& sl = L->slot[it % Lane::kSlots];
      const long long b0 = pipe_from + it * batch;
      const int cnt = (int)std::min(batch, n_perm - b0);
      if (!sl.ev[0])
        for (cudaEvent_t& e : sl.ev) LCK(cudaEventCreate(&e));
      if (!sl.side) LCK(cudaStreamCreateWithFlags(&sl.side, cudaStreamNonBlocking));
      if (!sl.dCnt) LCK(cudaMalloc(&sl.dCnt, 256));
      int r = lane_grow(L, &sl.dX, &sl.xBytes, (size_t)cnt * xs * 2);
      if (!r) r = lane_grow(L, &sl.dRes, &sl.resBytes, (size_t)cnt * sizeof(TaskResult));
      if (!r) r = lane_grow_host(L, &sl.hRes, &sl.hResBytes, (size_t)cnt * sizeof(TaskResult));
      if (!r) r = lane_grow(L, &sl.dFall, &sl.fallBytes, (size_t)3 * cnt * 4);
      if (r) return r;
      const int32_t* dI = nullptr;
      r = upload_idx(&sl.dIdx, &sl.idxBytes, b0, cnt, &dI);
      if (r) return r;
      NvtxRange range("dto: labels");
      LCK(cudaEventRecord(sl.ev[0], L->stream));
      r = make_labels_launch(L, P, seed, (uint32_t)(perm_first + b0), cnt, dI, (int16_t*)sl.dX, xs, true);
      if (r) return r;
      LCK(cudaEventRecord(sl.ev[1], L->stream));
      sl.b0 = b0;
      sl.cnt = cnt;
      return DTO_OK;
    };
    for (long long it = 0; it < std::min<long long>(npipe, 2); ++it) {
      rc = draw(it);
      if (rc) return rc;
      drawn[it] = true;
    }
    auto first_done = [&]() -> int {
      LCK(cudaEventSynchronize(L->evSide));
      float ms = 0.f;
      if (cnt0 > 0 && cudaEventElapsedTime(&ms, L->evk[0], L->evk[1]) == cudaSuccess) L->acc_perm_ms += ms;
      if (first_launch && cudaEventElapsedTime(&ms, L->evk[2], L->evk[3]) == cudaSuccess) L->acc_grid_ms += ms;
      if (want0) {
        if (!valid(hRes[0])) return lane_err(L, DTO_ERR_CUDA, "unpermuted task: the search returned no grid cell");
        unperm = hRes[0];
      }
      return take(hRes + 1, 0, cnt0);
    };
    if (!warm) {
      rc = first_done();
      if (rc) return rc;
      ladder_of(std::vector<double>(minp.begin(), minp.begin() + cnt0), P->fshift, tau);
    }
    if (pending) {
      ladder_flush(L->ctx, P);
      std::lock_guard<std::mutex> g(P->ladder_mu);
      for (int l = 0; l < kLadderTaus; ++l) tau[l] = P->ladder_tau[l];
    }
    if (model_later) {
      // the record (or, if another call recorded it meanwhile, the model's
      // entry); failing both, bounds below every cell leave each task to
      // the exhaustive screen (the same results, slowly)
      if (!ladder_take_deferred(L->ctx, shape_of(P), model_nats, &model_q0) &&
          !L->ctx->ladders.lookup(shape_of(P), model_nats, &model_q0)) {
        for (double& v : model_nats) v = -1.0e9;
        model_q0 = 0.0;
      }
      from_model();
    }
    // The table screens: the first sweep cascades through every level, so
    // it needs all of them.  They are built on the table stream, beside the
    // permutation kernel (a build block fits in what its CTAs leave of an
    // SM), after the main stream's work from before this run (the lane's
    // earlier sweeps read the same buffers), and the main stream's first
    // sweep waits for them.
    const int tight_levels = std::min(n_perm >= kTightAllMin ? kTightLevels : 0, kLadderLevels);
    bool built = false;
    for (int l = 0; l < kLadderLevels; ++l) {
      rc = ensure_table(L, P, l, tau[l], L->tstream, &built);
      if (rc) return rc;
    }
    for (int l = 0; l < tight_levels; ++l)
      for (int q = 0; q < kTightTables; ++q) {
        rc = ensure_table(L, P, tight_slot(l, q), tau[tight_slot(l, q)], L->tstream, &built);
        if (rc) return rc;
      }
    if (built) {
      LCK(cudaEventRecord(L->evTab, L->tstream));
      LCK(cudaStreamWaitEvent(L->stream, L->evTab, 0));
    }
    const int nlev = kLadderLevels;
    // Batches in flight: while batch b's exhaustive fallback and result copy
    // run on its slot's side stream, the next batches' labels and table
    // sweeps run on the main stream.
    auto harvest = [&](BatchSlot& sl) -> int {
      NvtxRange range("dto: result copy");
      LCK(cudaEventSynchronize(sl.ev[7]));
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, sl.ev[0], sl.ev[1]) == cudaSuccess) L->acc_perm_ms += ms;
      if (cudaEventElapsedTime(&ms, sl.ev[2], sl.ev[6]) == cudaSuccess) {
        L->acc_grid_ms += ms;
        L->acc_sweep0_ms += ms;
        L->acc_sweep0_launches += 1;
        L->acc_sweep0_tasks += sl.cnt;
      }
      if (cudaEventElapsedTime(&ms, sl.ev[4], sl.ev[5]) == cudaSuccess) L->acc_grid_ms += ms;
      const int trc = take((const TaskResult*)sl.hRes, sl.b0, sl.cnt);
      if (trc) return trc;
      L->acc_d2h += (long long)sl.cnt * (long long)sizeof(TaskResult);
      sl.busy = false;
      return DTO_OK;
    };
    for (long long it = 0; it < npipe; ++it) {
      if ((rc = cancelled())) return rc;
      BatchSlot& sl = L->slot[it % Lane::kSlots];
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
      LCK(cudaEventRecord(sl.ev[2], L->stream));
      rc = table_levels(L, P, X, xs, cnt, dR, (int*)sl.dFall, sl.dCnt, L->stream, 0, tight_levels);
      if (rc) return rc;
      LCK(cudaEventRecord(sl.ev[6], L->stream));
      last_l0_end = sl.ev[6];
      LCK(cudaStreamWaitEvent(sl.side, sl.ev[6], 0));
      LCK(cudaEventRecord(sl.ev[4], sl.side));
      rc = table_exhaustive(L, P, X, xs, cnt, dR, nlev, (const int*)sl.dFall, sl.dCnt, sl.side);
      if (rc) return rc;
      LCK(cudaEventRecord(sl.ev[5], sl.side));
      LCK(cudaMemcpyAsync(sl.hRes, dR, (size_t)cnt * sizeof(TaskResult), cudaMemcpyDeviceToHost, sl.side));
      LCK(cudaEventRecord(sl.ev[7], sl.side));
      sl.busy = true;
    }
    // the batches still in flight, oldest first: the host takes each one's
    // results while the later ones still run
    {
      BatchSlot* order[Lane::kSlots];
      int nb = 0;
      for (BatchSlot& sl : L->slot)
        if (sl.busy) order[nb++] = &sl;
      for (int x = 1; x < nb; ++x)  // at most kSlots entries, oldest first
        for (int y = x; y > 0 && order[y]->b0 < order[y - 1]->b0; --y) std::swap(order[y], order[y - 1]);
      for (int k = 0; k < nb; ++k) {
        rc = harvest(*order[k]);
        if (rc) return rc;
      }
    }
    if (warm) {
      rc = first_done();
      if (rc) return rc;
    }
    // this run's minimum p-values set the ladder of the pair's next run
    // (they are screens: any bounds give the same results).  On the
    // context's own lane the bounds are left to the next reader, which is
    // most often the pair's next run: it computes them while its labels are
    // drawn instead of this run's caller waiting for them.
    ladder_update(L->ctx, P, minp, L == L->ctx->lane0);
    // the main stream's timing event follows the side streams' last work
    LCK(cudaEventRecord(L->evSide, L->side));
    LCK(cudaStreamWaitEvent(L->stream, L->evSide, 0));
    for (BatchSlot& sl : L->slot) {
      if (!sl.side) continue;
      LCK(cudaEventRecord(sl.ev[3], sl.side));
      LCK(cudaStreamWaitEvent(L->stream, sl.ev[3], 0));
    }
  }
  long long count_le = -1;
  if (want0) {
    fill_result(P, unperm, 0, out_unpermuted);
    ++nroute[(unperm.route >= 0 && unperm.route < DTO_ROUTES) ? unperm.route : DTO_ROUTE_NONE];
    const double p_obs = unperm.p;
    count_le = 0;
    for (long long q = 0; q < n_perm; ++q) count_le += (minp[(size_t)q] <= p_obs);
  }
  LCK(cudaEventRecord(L->ev1, L->stream));
  unsigned long long refined[3] = {0, 0, 0};
  LCK(cudaMemcpyAsync(refined, L->dRefined, sizeof(refined), cudaMemcpyDeviceToHost, L->stream));
  LCK(cudaStreamSynchronize(L->stream));
  if (out_summary) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, L->ev0, L->ev1);
    dto_summary& s = *out_summary;
    s.n_perm = n_perm;
    s.count_le = count_le;
    if (want0) {
      s.empirical_pvalue = n_perm > 0 ? (double)count_le / (double)n_perm : 1.0;
      s.fdr = dto_fdr(out_unpermuted->set1_len, out_unpermuted->set2_len, out_unpermuted->intersection_size,
                      P->npop, 0.8);
    } else {
      s.empirical_pvalue = std::nan("");
      s.fdr = std::nan("");
    }
    s.logp_err_bound_screen = precision == DTO_PRECISION_SCREEN ? 4.5 * std::ldexp(1.0, -P->fshift) : 0.0;
    s.logp_err_bound_fp64 = 2.0e-13;
    s.n_fallback = (int64_t)refined[2];
    s.n_refined = (int64_t)refined[0];
    s.n_stage2 = (int64_t)refined[1];
    s.device_ms = ms;
    s.grid_ms = L->acc_grid_ms;
    s.perm_ms = L->acc_perm_ms;
    s.n_launches = L->acc_launches;
    s.h2d_bytes = L->acc_h2d;
    s.d2h_bytes = L->acc_d2h + 16;
    s.sweep0_ms = L->acc_sweep0_ms;
    s.sweep0_launches = L->acc_sweep0_launches;
    s.sweep0_tasks = L->acc_sweep0_tasks;
    s.tail_ms = 0.0;
    if (last_l0_end && cudaEventElapsedTime(&ms, last_l0_end, L->ev1) == cudaSuccess) s.tail_ms = ms;
    for (int q = 0; q < DTO_ROUTES; ++q) s.n_route[q] = nroute[q];
  }
  return DTO_OK;
}

}  // namespace dto
