// dto_wave.cpp -- dto_batch_run's waves.
//
// A batch holds many short runs (config 3: 512 pairs of 10,000
// permutations).  Run one by one, each pair's cascade sweep is a launch of its
// own, and every launch ends in a tail in which the last tasks hold a few SMs
// while the rest idle: at N = 20,000 a 10,000-task launch costs about 2.5
// times what its tasks cost inside a long launch.  A wave instead draws the
// labels of several pairs, then sweeps all their tasks in one launch of
// table_hw_kernel's multi-pair mode (one segment per pair), so only the wave
// has a tail.  Each pair keeps its own ladder and table screens (built into
// buffers the pair owns, so that the next batch finds them), its unpermuted
// task goes through the exhaustive screen on the side stream as in a lane's
// run, and its exhaustive fallbacks follow the sweep.  The searches are the
// same as a lane's, so the results are the same bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "dto_host.h"

namespace dto {

namespace {

constexpr int64_t kWaveMinPerm = 1025;   // shorter runs: the exhaustive screen (a lane's run)
constexpr int64_t kWaveMaxPerm = 32767;  // longer runs: a lane's pipeline with its tighter tables
constexpr size_t kWaveLabelBytes = size_t(8) << 30;  // labels of one wave (two in flight)
constexpr int kWaveLevels = 3;

// The pair's ladder (levels 0..2): its own from an earlier run, else the
// context's model's for its shape.
bool wave_taus(dto_ctx* ctx, dto_pair* P, int tau[kLadderTaus]) {
  ladder_flush(ctx, P);
  {
    std::lock_guard<std::mutex> g(P->ladder_mu);
    if (P->ladder_ok) {
      for (int l = 0; l < kLadderTaus; ++l) tau[l] = P->ladder_tau[l];
      return true;
    }
  }
  ladder_flush_deferred(ctx);
  double nats[kLadderTaus], q0 = 0.0;
  if (!ctx->ladders.lookup(shape_of(P), nats, &q0)) return false;
  {
    std::lock_guard<std::mutex> g(P->ladder_mu);
    if (P->q0 <= 0.0) P->q0 = q0;
  }
  const double scale = std::ldexp(1.0, P->fshift);
  for (int l = 0; l < kLadderTaus; ++l) tau[l] = (int)std::max(-2.0e9, std::min(0.0, std::floor(nats[l] * scale)));
  ladder_order(tau);
  return true;
}

// The pair's table screen of `level` for bound tau, built on the lane's main
// stream unless the pair already holds it.
int wave_table(Lane* L, dto_pair* P, int level, int tau, long long* launches) {
  if (P->wave_ok[level] && P->wave_tau[level] == tau) return DTO_OK;
  if (!P->dWaveKthr[level]) {
    const size_t bytes = table_entries(P->C, P->dev.n1) * 2;
    if (cudaMalloc(&P->dWaveKthr[level], bytes) != cudaSuccess) {
      cudaGetLastError();
      P->dWaveKthr[level] = nullptr;
      return lane_err(L, DTO_ERR_OOM, "out of device memory for a pair's table screen");
    }
  }
  TableArgs t{};
  t.n1 = P->dev.n1;
  t.n2 = P->dev.n2;
  t.N = (int)P->npop;
  t.C = 2 * P->C;  // the half-warp sweep's 16 lanes of 2 C columns
  t.rowstart = P->dRow;
  t.ncnt = P->dNcnt;
  t.F = P->dF;
  t.fshift = P->fshift;
  t.tau = tau;
  t.mcnt = P->dMcnt;
  t.N1 = (int)P->N1;
  t.kthr = P->dWaveKthr[level];
  P->wave_ok[level] = false;
  LCK(launch_table_build(t, L->ctx->nsm, L->stream));
  P->wave_tau[level] = tau;
  P->wave_ok[level] = true;
  *launches += 1;
  return DTO_OK;
}

// A wave in flight: its jobs, its buffers and its layout.
struct Wave {
  std::vector<int> w;  // indices into the jobs
  Lane::WaveBuf* buf = nullptr;
  std::vector<long long> roff;
  std::vector<long long> launches;
  long long rtot = 0;
};

// Enqueues wave `wv` on the lane's streams: the pairs' table screens and
// labels, their unpermuted tasks (side stream), the multi-pair sweep, the
// exhaustive fallbacks and the copy of the results.
int enqueue_wave(Lane* L, std::vector<WaveJob>& jobs, Wave& wv) {
  dto_ctx* ctx = L->ctx;
  Lane::WaveBuf& B = *wv.buf;
  const int nj = (int)wv.w.size();
  const int C = jobs[(size_t)wv.w[0]].P->C;
  auto job = [&](int k) -> WaveJob& { return jobs[(size_t)wv.w[(size_t)k]]; };
  // per job: its labels (row 0: the unpermuted task), its results, its
  // fallback lists (three of n_perm entries), 16 counters, 4 refine counts
  std::vector<long long> xoff((size_t)nj), foff((size_t)nj);
  wv.roff.assign((size_t)nj, 0);
  wv.launches.assign((size_t)nj, 0);
  long long xtot = 0, rtot = 0, ftot = 0;
  for (int k = 0; k < nj; ++k) {
    xoff[(size_t)k] = xtot;
    wv.roff[(size_t)k] = rtot;
    foff[(size_t)k] = ftot;
    xtot += (job(k).n_perm + 1) * xstride_of(job(k).P->N1);
    rtot += job(k).n_perm + 1;
    ftot += 3 * job(k).n_perm;
  }
  wv.rtot = rtot;
  const size_t cnt_bytes = (size_t)nj * 16 * 4, ref_bytes = (size_t)nj * 4 * 8;
  int rc = lane_grow(L, &B.dX, &B.xBytes, (size_t)xtot * 2);
  if (!rc) rc = lane_grow(L, &B.dRes, &B.resBytes, (size_t)rtot * sizeof(TaskResult));
  if (!rc) rc = lane_grow_host(L, &B.hRes, &B.hResBytes, (size_t)rtot * sizeof(TaskResult) + ref_bytes);
  if (!rc) rc = lane_grow(L, &B.dAux, &B.auxBytes, cnt_bytes + ref_bytes + (size_t)ftot * 4);
  if (!rc) rc = lane_grow(L, &B.dSegs, &B.segsBytes, (size_t)nj * sizeof(TableGridArgs));
  if (!rc) rc = lane_grow_host(L, &B.hSegs, &B.hSegsBytes, (size_t)nj * sizeof(TableGridArgs));
  if (!rc)
    rc = lane_grow(L, &L->dHits[0], &L->hitBytes[0],
                   (size_t)kTableCtasPerSm * ctx->nsm * kTableWarps * kTableWarpHits * 8);
  if (rc) return rc;
  for (cudaEvent_t& e : B.ev)
    if (!e) LCK(cudaEventCreate(&e));
  int16_t* X = (int16_t*)B.dX;
  TaskResult* dRes = (TaskResult*)B.dRes;
  int* cnts = (int*)B.dAux;
  unsigned long long* refined = (unsigned long long*)((char*)B.dAux + cnt_bytes);
  int* fall = (int*)((char*)B.dAux + cnt_bytes + ref_bytes);
  NvtxRange range("dto: wave");
  LCK(cudaEventRecord(B.ev[0], L->stream));
  LCK(cudaMemsetAsync(B.dAux, 0, cnt_bytes + ref_bytes, L->stream));
  // the pairs' table screens, then their labels (permutations 1..n_perm)
  for (int k = 0; k < nj; ++k)
    for (int l = 0; l < kWaveLevels; ++l) {
      rc = wave_table(L, job(k).P, l, job(k).tau[l], &wv.launches[(size_t)k]);
      if (rc) return rc;
    }
  {
    NvtxRange lr("dto: labels");
    for (int k = 0; k < nj; ++k) {
      const long long xs = xstride_of(job(k).P->N1);
      rc = make_labels_launch(L, job(k).P, job(k).seed, job(k).first, (int)job(k).n_perm, nullptr,
                              X + xoff[(size_t)k] + xs, xs, true);
      if (rc) return rc;
      wv.launches[(size_t)k] += 1;
    }
  }
  LCK(cudaEventRecord(B.ev[1], L->stream));
  // the unpermuted tasks: row 0 of each job, the exhaustive screen with a
  // CTA per task, on the side stream beside the sweep (after the previous
  // wave's, whose buffers these are not)
  for (int k = 0; k < nj; ++k) {
    const long long xs = xstride_of(job(k).P->N1);
    LCK(cudaMemcpyAsync(X + xoff[(size_t)k], job(k).P->dYlab, (size_t)job(k).P->N1 * 2, cudaMemcpyDeviceToDevice,
                        L->side));
    rc = lane_grid_tasks(L, job(k).P, X + xoff[(size_t)k], xs, 1, kModeScreen, dRes + wv.roff[(size_t)k], nullptr,
                         nullptr, false, L->side, true);
    if (rc) return rc;
    wv.launches[(size_t)k] += 1;
  }
  LCK(cudaEventRecord(L->evSide, L->side));
  // one segment per job: the arguments of its cascade sweep
  TableGridArgs* hs = (TableGridArgs*)B.hSegs;
  long long ntot = 0;
  for (int k = 0; k < nj; ++k) {
    dto_pair* P = job(k).P;
    const long long xs = xstride_of(P->N1);
    const long long cap = job(k).n_perm;
    TableGridArgs a{};
    a.P = P->dev;
    a.P.LF = ctx->dLF.load();
    a.X = X + xoff[(size_t)k] + xs;
    a.xstride = xs;
    a.ntask = (int)job(k).n_perm;
    a.tau = job(k).tau[0];
    a.kthr = P->dWaveKthr[0];
    a.ntight = 0;
    a.nlev = kWaveLevels;
    for (int l = 1; l < kWaveLevels; ++l) {
      a.kthr_up[l - 1] = P->dWaveKthr[l];
      a.tau_up[l - 1] = job(k).tau[l];
      a.ntight_up[l - 1] = 0;
    }
    a.route = DTO_ROUTE_LEVEL0;
    a.smemF = 0;
    a.out = dRes + wv.roff[(size_t)k] + 1;
    a.work = cnts + 16 * k;
    a.n_refined = refined + 4 * k;
    a.fallback = fall + foff[(size_t)k] + (kWaveLevels - 1) * cap;
    a.nfallback = cnts + 16 * k + 8 + kWaveLevels - 1;
    a.hitbuf = (int2*)L->dHits[0];
    a.hitcap = kTableWarpHits;
    hs[k] = a;
    ntot += job(k).n_perm;
  }
  LCK(cudaMemcpyAsync(B.dSegs, hs, (size_t)nj * sizeof(TableGridArgs), cudaMemcpyHostToDevice, L->stream));
  {
    NvtxRange sr("dto: wave sweep");
    TableGridArgs la{};
    la.P = job(0).P->dev;
    la.hitbuf = (int2*)L->dHits[0];
    la.hitcap = kTableWarpHits;
    la.segs = (const TableGridArgs*)B.dSegs;
    la.nseg = nj;
    const int ctas = (int)std::max(1LL, std::min<long long>((long long)kTableCtasPerSm * ctx->nsm,
                                                          ntot / (kTableWarps * 2) + 1));
    LCK(launch_table_grid(la, C, ctas, L->stream));
    wv.launches[0] += 1;
  }
  LCK(cudaEventRecord(B.ev[2], L->stream));
  // what the last level left, per job
  for (int k = 0; k < nj; ++k) {
    const long long xs = xstride_of(job(k).P->N1);
    rc = table_exhaustive(L, job(k).P, X + xoff[(size_t)k] + xs, xs, (int)job(k).n_perm,
                          dRes + wv.roff[(size_t)k] + 1, kWaveLevels, fall + foff[(size_t)k], cnts + 16 * k, L->stream,
                          refined + 4 * k);
    if (rc) return rc;
    wv.launches[(size_t)k] += 1;
  }
  LCK(cudaStreamWaitEvent(L->stream, L->evSide, 0));
  LCK(cudaMemcpyAsync(B.hRes, dRes, (size_t)rtot * sizeof(TaskResult), cudaMemcpyDeviceToHost, L->stream));
  LCK(cudaMemcpyAsync((char*)B.hRes + (size_t)rtot * sizeof(TaskResult), refined, ref_bytes, cudaMemcpyDeviceToHost,
                      L->stream));
  LCK(cudaEventRecord(B.ev[3], L->stream));
  return DTO_OK;
}

// Waits for wave `wv` and hands each job its results, ladder and summary.
int finish_wave(Lane* L, std::vector<WaveJob>& jobs, Wave& wv) {
  dto_ctx* ctx = L->ctx;
  Lane::WaveBuf& B = *wv.buf;
  LCK(cudaEventSynchronize(B.ev[3]));
  float wave_ms = 0.f, label_ms = 0.f, sweep_ms = 0.f;
  cudaEventElapsedTime(&wave_ms, B.ev[0], B.ev[3]);
  cudaEventElapsedTime(&label_ms, B.ev[0], B.ev[1]);
  cudaEventElapsedTime(&sweep_ms, B.ev[1], B.ev[2]);
  const TaskResult* hRes = (const TaskResult*)B.hRes;
  const unsigned long long* hRef = (const unsigned long long*)((const char*)B.hRes + (size_t)wv.rtot * sizeof(TaskResult));
  for (int k = 0; k < (int)wv.w.size(); ++k) {
    WaveJob& j = jobs[(size_t)wv.w[(size_t)k]];
    dto_pair* P = j.P;
    const int nt1 = (int)P->T1.size(), nt2 = (int)P->T2.size();
    const TaskResult* hr = hRes + wv.roff[(size_t)k];
    for (long long q = 0; q <= j.n_perm; ++q) {
      const TaskResult& r = hr[q];
      if (!(r.i >= 0 && r.i < nt1 && r.j >= 0 && r.j < nt2)) {
        if (q == 0) return lane_err(L, DTO_ERR_CUDA, "unpermuted task: the search returned no grid cell");
        char msg[160];
        std::snprintf(msg, sizeof(msg), "permutation %lld: the search returned no grid cell", q);
        return lane_err(L, DTO_ERR_CUDA, msg);
      }
    }
    std::vector<double> minp((size_t)j.n_perm);
    long long nroute[DTO_ROUTES] = {};
    long long count_le = 0;
    const double p_obs = hr[0].p;
    for (long long q = 0; q < j.n_perm; ++q) {
      const TaskResult& r = hr[q + 1];
      minp[(size_t)q] = r.p;
      count_le += (r.p <= p_obs);
      ++nroute[(r.route >= 0 && r.route < DTO_ROUTES) ? r.route : DTO_ROUTE_NONE];
    }
    ++nroute[(hr[0].route >= 0 && hr[0].route < DTO_ROUTES) ? hr[0].route : DTO_ROUTE_NONE];
    if (j.out_minp) std::memcpy(j.out_minp, minp.data(), (size_t)j.n_perm * sizeof(double));
    fill_result(P, hr[0], 0, j.out_unpermuted);
    ladder_update(ctx, P, minp);
    if (j.out_summary) {
      // a wave's times are shared by its jobs in proportion to their tasks
      const double share = (double)(j.n_perm + 1) / (double)wv.rtot;
      dto_summary& s = *j.out_summary;
      s = dto_summary{};
      s.n_perm = j.n_perm;
      s.count_le = count_le;
      s.empirical_pvalue = j.n_perm > 0 ? (double)count_le / (double)j.n_perm : 1.0;
      s.fdr = dto_fdr(j.out_unpermuted->set1_len, j.out_unpermuted->set2_len, j.out_unpermuted->intersection_size,
                      P->npop, 0.8);
      s.logp_err_bound_screen = 4.5 * std::ldexp(1.0, -P->fshift);
      s.logp_err_bound_fp64 = 2.0e-13;
      s.n_fallback = (int64_t)hRef[4 * k + 2];
      s.n_refined = (int64_t)hRef[4 * k];
      s.n_stage2 = (int64_t)hRef[4 * k + 1];
      s.device_ms = wave_ms * share;
      s.grid_ms = sweep_ms * share;
      s.perm_ms = label_ms * share;
      s.n_launches = wv.launches[(size_t)k];
      s.h2d_bytes = (int64_t)sizeof(TableGridArgs);
      s.d2h_bytes = (int64_t)((j.n_perm + 1) * (long long)sizeof(TaskResult) + 32);
      s.sweep0_ms = sweep_ms * share;
      s.sweep0_launches = k == 0 ? 1 : 0;
      s.sweep0_tasks = j.n_perm;
      s.tail_ms = 0.0;
      for (int q = 0; q < DTO_ROUTES; ++q) s.n_route[q] = nroute[q];
    }
  }
  return DTO_OK;
}

}  // namespace

long long wave_label_bytes(const dto_pair* P, int64_t n_perm) { return (n_perm + 1) * xstride_of(P->N1) * 2; }

bool wave_eligible(dto_ctx* ctx, dto_pair* P, int64_t n_perm, int precision) {
  if (!ctx || !P || P->ctx != ctx) return false;
  if (precision != DTO_PRECISION_SCREEN || !P->same_set) return false;
  if (n_perm < kWaveMinPerm || n_perm > kWaveMaxPerm) return false;
  int tau[kLadderTaus];
  return wave_taus(ctx, P, tau);
}

int lane_wave(Lane* L, std::vector<WaveJob>& jobs) {
  if (jobs.empty()) return DTO_OK;
  LCK(cudaSetDevice(L->ctx->device));
  for (WaveJob& j : jobs) {
    int tau[kLadderTaus];
    if (!wave_taus(L->ctx, j.P, tau)) return lane_err(L, DTO_ERR_INVALID, "a wave's pair has no ladder");
    for (int l = 0; l < kWaveLevels; ++l) j.tau[l] = tau[l];
  }
  // waves of one C each, in the order the jobs came, while their labels fit
  std::vector<int> order(jobs.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[(size_t)a].P->C < jobs[(size_t)b].P->C; });
  std::vector<Wave> waves;
  for (size_t q = 0; q < order.size();) {
    const int C = jobs[(size_t)order[q]].P->C;
    Wave wv;
    size_t bytes = 0;
    while (q < order.size() && jobs[(size_t)order[q]].P->C == C) {
      const WaveJob& j = jobs[(size_t)order[q]];
      const size_t b = (size_t)wave_label_bytes(j.P, j.n_perm);
      if (!wv.w.empty() && bytes + b > kWaveLabelBytes) break;
      wv.w.push_back(order[q]);
      bytes += b;
      ++q;
    }
    waves.push_back(std::move(wv));
  }
  // two waves in flight: the host takes one wave's results while the next
  // runs (each wave's buffers are reused two waves later, after the host
  // has taken its results)
  for (size_t k = 0; k < waves.size(); ++k) {
    waves[k].buf = &L->wave[k % 2];
    int rc = enqueue_wave(L, jobs, waves[k]);
    if (!rc && k > 0) rc = finish_wave(L, jobs, waves[k - 1]);
    if (rc) {
      cudaStreamSynchronize(L->stream);
      cudaStreamSynchronize(L->side);
      return rc;
    }
  }
  const int rc = finish_wave(L, jobs, waves.back());
  return rc;
}

}  // namespace dto
