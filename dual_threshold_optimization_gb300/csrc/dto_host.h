// dto_host.h -- host-side state of libdto.so shared by the C ABI
// (dto_capi.cpp), the permutation-null driver (dto_lane.cpp) and the
// request executor (dto_serve.cpp).
//
// A context owns the device, the shared log-factorial table and one default
// lane.  A lane is everything one run of the permutation null needs while it
// is in flight: two streams, events, scratch buffers and the table screens of
// the pair it last ran.  dto_run and the other context-level calls use the
// default lane under the context's mutex; an executor owns further lanes and
// runs one request on each at a time, so that requests overlap on the device.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/dto.h"
#include "dto_internal.h"

namespace dto {

// An NVTX range over a stage of a run (header-only NVTX: without a profiler
// attached the push and pop cost a branch).  The ranges mark the host-side
// enqueue of each stage; the device work follows on the lane's streams.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

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
  cudaEvent_t ev[8] = {};  // perm start/end, tables start, side drained, exhaustive start/end, tables done, batch done
  // the stream of this slot's later table levels, fallbacks and result copy:
  // the side work of different batches overlaps (each is latency-bound)
  cudaStream_t side = nullptr;
  bool busy = false;
  long long b0 = 0;
  int cnt = 0;
};

constexpr int kSlotsMax = 4;

// The ladder's fixed-point bounds: levels 0..2, then three tighter tables
// per level.
constexpr int kLadderTaus = 12;
constexpr int tight_slot(int level, int q) { return 3 + 3 * level + q; }

struct Lane {
  dto_ctx* ctx = nullptr;
  // set by a server's worker to its request's cancel flag: a run checks it
  // between batches and returns DTO_ERR_CANCELLED once its work in flight
  // has drained (kernels are never interrupted)
  std::atomic<int>* cancel = nullptr;
  std::string* err = nullptr;  // where this lane's error messages go
  std::string own_err;
  // first batch with a CTA per task: lowest latency for a run alone; lanes
  // that share the GPU with other runs take the warp-per-task screen, whose
  // throughput is higher
  bool coop_first = true;
  // a pair without a ladder of its own starts from the ladder of an earlier
  // pair of the same shape (LadderModel), skipping its first batch (every
  // lane of a context and its servers)
  bool use_model = false;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // first batch, unpermuted task, fallbacks
  cudaStream_t tstream = nullptr;  // a run's table screens, beside its labels
  cudaEvent_t evTab = nullptr;     // the table screens built
  cudaEvent_t evSide = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t evk[4] = {nullptr, nullptr, nullptr, nullptr};  // perm start/end, grid start/end
  // per-run accounting
  double acc_grid_ms = 0.0, acc_perm_ms = 0.0, acc_sweep0_ms = 0.0;
  long long acc_launches = 0, acc_h2d = 0, acc_d2h = 0, acc_sweep0_launches = 0, acc_sweep0_tasks = 0;
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
  // per-warp hit buffers of the table sweep (main stream)
  void* dHits[1] = {};
  size_t hitBytes[1] = {};
  // Batches of the table-screen pipeline in flight.  A slot is reused only
  // once its side stream has finished its batch (fallbacks, result copy);
  // with three, the main stream draws the next batch's labels while a side
  // stream still finishes the batch before last.
  static constexpr int kSlots = 3;
  static_assert(kSlots >= 2 && kSlots <= kSlotsMax, "two to four batch slots");
  BatchSlot slot[kSlots];
  // table screens of the pair this lane last ran: the ladder's levels 0..2,
  // then three tighter tables per level (tight_slot) that a sweep switches
  // to once a task's bound is known
  static constexpr int kTables = kLadderTaus;
  uint16_t* dKthr[kTables] = {};
  size_t kthrBytes[kTables] = {};
  unsigned long long kthr_pair[kTables] = {};  // pair serial the table was built for (0: none)
  int kthr_tau[kTables] = {};
  // dto_batch_run's waves (lane_wave), two in flight: labels, results,
  // fallback lists and counters, and the segment arguments of the
  // multi-pair sweep
  struct WaveBuf {
    void* dX = nullptr;
    size_t xBytes = 0;
    void* dRes = nullptr;
    size_t resBytes = 0;
    void* hRes = nullptr;  // pinned
    size_t hResBytes = 0;
    void* dAux = nullptr;
    size_t auxBytes = 0;
    void* dSegs = nullptr;
    size_t segsBytes = 0;
    void* hSegs = nullptr;  // pinned
    size_t hSegsBytes = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // start, labels done, sweep done, end
  };
  WaveBuf wave[2];
  std::vector<double> minp;  // a run's minimum p-values (lane_run_range)
};

// Ladders of the pairs a context has run, by shape, in nats of ln p.  The
// null distribution of the minimum p-value depends on the pair's shape (list
// lengths, shared features, population, grid) and hardly on its ranks, and a
// ladder decides only which path settles each permutation, never a result:
// so a pair of nearly the same shape as an earlier one can start from that
// pair's ladder instead of measuring its own from an exhaustive first batch.
struct LadderShape {
  long long npop, N1, N2, ncommon;
  int n1, n2;
  bool same_set;
  double nats[kLadderTaus];
  double q0;  // the level-0 quantile the ladder was built with
};

// A run's minimum p-values not yet made into ladder bounds: the context's
// own lane leaves that work to the pair's next reader (its next run computes
// the bounds while its labels are drawn).  The context keeps a copy of the
// last one for its model, so that a new pair of the same shape finds it even
// if its pair never runs again.
struct LadderPending {
  std::vector<double> sample;  // evenly strided, at most 16,384 minima
  double pmax = 0.0;           // the largest of all the run's minima
  double q0 = 0.0;             // the level-0 quantile
  int fshift = 0;
  LadderShape shape{};         // nats unset
  unsigned long long serial = 0, gen = 0;  // the pair and its update
};

struct LadderModel {
  std::mutex mu;
  std::vector<LadderShape> shapes;  // most recent last
  static constexpr size_t kMaxShapes = 4096;
  static constexpr double kTol = 0.05;  // relative difference accepted per size
  void record(const LadderShape& x);
  bool lookup(const LadderShape& want, double nats[kLadderTaus], double* q0 = nullptr);
  // x stands in for want: the same kind of lists, every size within kTol
  // (their relative differences' sum in *dist)
  static bool fits(const LadderShape& x, const LadderShape& want, double* dist = nullptr);
};

}  // namespace dto

struct dto_ctx {
  int device = 0;
  int nsm = 0;
  size_t smem_optin = 0;  // dynamic shared-memory budget of one block
  std::string err;
  std::mutex mu;       // serialises the context-level calls (default lane, pair creation)
  std::mutex lf_mu;    // guards the log-factorial table
  // ln(m!) as double-double, m = 0..lf_cap; a grown table replaces the old
  // one, which stays allocated until the context is destroyed (kernels of
  // other lanes may still read it)
  long long lf_cap = -1;
  std::vector<double> lf_hi, lf_lo;
  std::atomic<double2*> dLF{nullptr};
  std::vector<double2*> lf_old;
  std::atomic<unsigned long long> next_serial{1};
  dto::Lane* lane0 = nullptr;
  dto::LadderModel ladders;
  // the last run of the context's own lane whose ladder is pending: recorded
  // into `ladders` when a new pair looks its shape up, unless its pair's own
  // next reader has done so
  std::mutex defer_mu;
  bool deferred = false;
  dto::LadderPending deferred_rec;
};

struct dto_pair {
  dto_ctx* ctx = nullptr;
  unsigned long long serial = 0;  // unique per context: keys the lanes' table caches
  uint32_t pair_id = 0;
  long long N1 = 0, N2 = 0, npop = 0, nfeat = 0, ncommon = 0;
  bool same_set = false;
  std::vector<uint32_t> r1, r2, T1, T2;
  std::vector<int32_t> order1, order2, f1, f2;
  std::vector<int> c1, c2, map12;
  std::vector<int16_t> lab2, ylab;
  int C = 0, fshift = 0;
  long long upload_bytes = 0;  // host-to-device bytes of dto_pair_create
  // device: views into one allocation (dBase)
  void* dBase = nullptr;
  int* dRow = nullptr;
  int* dNcnt = nullptr;
  uint32_t* dF = nullptr;
  int16_t* dYlab = nullptr;
  int16_t* dLab2 = nullptr;
  int16_t* dYlabHw = nullptr;  // dYlab and dLab2 in the table sweep's label form
  int16_t* dLab2Hw = nullptr;
  int* dMap12 = nullptr;
  int* dMcnt = nullptr;  // [n2]: list-1 positions whose label's column is <= j
  dto::PairDev dev{};
  // The table ladder (fixed-point bounds of levels 0..2) from the last long
  // run of this pair: a property of the pair's null distribution, so a later
  // run starts its pipeline with it instead of measuring a first batch.
  std::mutex ladder_mu;
  bool ladder_ok = false;
  int ladder_tau[dto::kLadderTaus] = {};
  // the level-0 quantile of its ladder (0: the default, dto::kLevel0Quantile),
  // and an evenly strided sample of the last run's minimum p-values, from
  // which a new quantile rebuilds the ladder (dto_pair_set_level0_quantile)
  double q0 = 0.0;
  std::vector<double> ladder_sample;
  // ladder_sample (and the maximum) of the last run, not yet made into
  // bounds (ladder_flush); `ladder_gen` counts the pair's deferred updates
  bool ladder_pending = false;
  double ladder_pmax = 0.0;
  unsigned long long ladder_gen = 0;
  // The table screens of levels 0..2 that dto_batch_run's waves built for
  // this pair, kept with it (a wave sweeps several pairs at once, so each
  // needs its own; the next batch finds them).  Guarded by the context mutex.
  uint16_t* dWaveKthr[3] = {};
  int wave_tau[3] = {};
  bool wave_ok[3] = {};
};

namespace dto {

int set_err(dto_ctx* ctx, int code, const std::string& msg);
int cuda_err(dto_ctx* ctx, cudaError_t e, const char* what);
int lane_err(Lane* L, int code, const std::string& msg);
int lane_cuda_err(Lane* L, cudaError_t e, const char* what);

#define CK(call)                                                \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return dto::cuda_err(ctx, e_, #call); \
  } while (0)

#define LCK(call)                                                 \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return dto::lane_cuda_err(L, e_, #call); \
  } while (0)

int lane_create(dto_ctx* ctx, Lane** out, std::string* err_sink);
void lane_destroy(Lane* L);
int lane_grow(Lane* L, void** p, size_t* cap, size_t need);
int lane_grow_host(Lane* L, void** p, size_t* cap, size_t need);

long long xstride_of(long long N1);
int check_perm(const int32_t* idx, long long L);
void fill_result(const dto_pair* P, const TaskResult& r, int permuted, dto_result* o);

// One task per launch through the exhaustive screen (or FP64 / dump modes).
int lane_grid_tasks(Lane* L, dto_pair* P, const int16_t* dX, long long xstride, int ntask, int mode,
                    TaskResult* dOut, int* dumpK = nullptr, double* dumpP = nullptr, bool guess = false,
                    cudaStream_t stream = nullptr, bool coop = false);
// Labels of `count` permutations from perm id `first` (or of uploaded index
// rows dIdx) into L->dX from row `row0`.
int lane_make_labels(Lane* L, dto_pair* P, uint64_t seed, uint32_t first, int count, const int32_t* dIdx,
                     int row0 = 0);

// The permutation null of one pair on one lane (dto_run_range's semantics).
// `minp` receives every permutation's minimum p (n_perm entries).
int lane_run_range(Lane* L, dto_pair* P, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                   const int32_t* perm_idx, int precision, dto_result* out_unpermuted, double* out_minp,
                   dto_result* out_perm, dto_summary* out_summary);

// The table ladder's bounds (fixed-point ln p, kLadderTaus of them) from a
// sample of minimum p-values, in ladder order.
void ladder_of(const std::vector<double>& all, int fshift, int tau[kLadderTaus], double q0 = 0.0);
// The default level-0 quantile (a pair's own, or a tuned one, replaces it).
extern const double kLevel0QuantileDefault;
void ladder_order(int tau[kLadderTaus]);
LadderShape shape_of(const dto_pair* P);
// A run's ladder after it: bounds that moved by more than the slack replace
// the pair's, and the context's model records the pair's shape.  With
// `defer` the bounds are left pending for the pair's next reader.
void ladder_update(dto_ctx* ctx, dto_pair* P, const std::vector<double>& minp, bool defer = false);
// The pair's pending ladder made into bounds (nothing if none is pending).
void ladder_flush(dto_ctx* ctx, dto_pair* P);
// The context's pending record made into its model's entry.
void ladder_flush_deferred(dto_ctx* ctx);
// Does the context's pending record fit a pair of shape `want`?
bool ladder_deferred_fits(dto_ctx* ctx, const LadderShape& want);
// The context's pending record, if it fits `want`, made into its model's
// entry; its bounds (nats) and level-0 quantile returned.
bool ladder_take_deferred(dto_ctx* ctx, const LadderShape& want, double nats[kLadderTaus], double* q0);
// Labels of `count` permutations from perm id `first` (or of uploaded index
// rows dIdx) into X (row stride xs) on the lane's main stream.
int make_labels_launch(Lane* L, dto_pair* P, uint64_t seed, uint32_t first, int count, const int32_t* dIdx,
                       int16_t* X, long long xs, bool hwlab = false);
// The exhaustive screen of what the last table level left, on `stream`.
int table_exhaustive(Lane* L, dto_pair* P, const int16_t* X, long long xstride, int ntask, TaskResult* dOut,
                     int nlev, const int* fall, int* cnts, cudaStream_t stream,
                     unsigned long long* refined = nullptr);

// One pair's run inside a wave of dto_batch_run.
struct WaveJob {
  dto_pair* P = nullptr;
  uint32_t first = 1;  // permutation ids first .. first + n_perm - 1
  int64_t n_perm = 0;
  uint64_t seed = 0;
  dto_result* out_unpermuted = nullptr;
  double* out_minp = nullptr;  // nullable
  dto_summary* out_summary = nullptr;  // nullable
  int tau[3] = {};  // the levels' bounds (set by lane_wave)
};
// Runs that a wave takes: the screen, lists over one feature set,
// kWaveMinPerm..kWaveMaxPerm permutations, and a ladder (the pair's own, or
// the context's model's).
bool wave_eligible(dto_ctx* ctx, dto_pair* P, int64_t n_perm, int precision);
// Device bytes of labels a wave holds for a job.
long long wave_label_bytes(const dto_pair* P, int64_t n_perm);
// The runs of `jobs` (all eligible) in waves: per
// wave the pairs' labels, then one cascade sweep over all their tasks, then
// their exhaustive fallbacks; each pair's unpermuted task through the
// exhaustive screen on the side stream.  The results equal lane_run_range's
// bit for bit.  Returns the first failure.
int lane_wave(Lane* L, std::vector<WaveJob>& jobs);

// Bytes of device scratch a run of the pair holds at its peak (labels of the
// batches in flight, results, hit buffers, table screens).
long long run_device_bytes(const dto_ctx* ctx, const dto_pair* P, int64_t n_perm, bool test_mode);

}  // namespace dto
