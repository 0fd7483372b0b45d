/*
 * dto.h -- C ABI of the GB300 Dual Threshold Optimization engine (libdto.so).
 *
 * Plain pointers and sizes only.  Every entry point returns a status code
 * (DTO_OK on success); dto_last_error() gives the message of the last failure
 * on a context.  Each declaration names the reference interface it replaces
 * (paths relative to the reference project).
 *
 * Vocabulary:
 *   list        a ranked feature list: (rank, feature id) per feature.  Feature
 *               ids are dense integers in [0, n_features) shared by both lists.
 *   position    index into a list after the stable sort by rank
 *               (src/collections/ranked.rs:527-542).
 *   thresholds  the reference's grid T1 = 1, T(k+1) = floor(T(k)*1.01 + 1) while
 *               T <= max rank (src/collections/ranked.rs:359-375).
 *   cell        one (threshold1, threshold2) pair of the grid.
 *   task        one optimize() call: the unpermuted task or one permutation
 *               (src/run/task.rs:3-9).
 */
#ifndef DTO_H
#define DTO_H

#include <stdint.h>

#if defined(__GNUC__)
#define DTO_API __attribute__((visibility("default")))
#else
#define DTO_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define DTO_OK 0
#define DTO_ERR_INVALID 1  /* bad arguments; the reference panics in these cases */
#define DTO_ERR_OOM 2      /* device or host allocation failed */
#define DTO_ERR_TIMEOUT 3  /* a bounded wait (dto_serve_wait_for) ran out first */
#define DTO_ERR_CUDA 4     /* any other CUDA runtime failure */
#define DTO_ERR_NOT_FOUND 5
#define DTO_ERR_CANCELLED 6 /* the request was cancelled (dto_serve_cancel) */

/* Precision of the threshold-pair search. */
#define DTO_PRECISION_FP64 0   /* plain FP64: the FP64 tail of every cell (drop-in path) */
#define DTO_PRECISION_SCREEN 1 /* 32-bit log-space screen of every cell, FP64 refine of the
                                  cells within the proven margin; same argmin, same p */

/* Which search path settled a task (dto_result.route).  Every path returns the
 * same optimum; the code says only which one did the work. */
#define DTO_ROUTE_NONE 0      /* not recorded */
#define DTO_ROUTE_SCREEN 1    /* exhaustive screen: short runs of a pair without a ladder, a long run's first batch, task 0 */
#define DTO_ROUTE_LEVEL0 2    /* table screen, level 0 of the ladder */
#define DTO_ROUTE_LEVEL1 3    /* table screen, level 1 */
#define DTO_ROUTE_LEVEL2 4    /* table screen, level 2 */
#define DTO_ROUTE_FALLBACK 5  /* exhaustive screen of a task no table level settled */
#define DTO_ROUTE_FP64 6      /* plain FP64 path (DTO_PRECISION_FP64) */
#define DTO_ROUTES 8

typedef struct dto_ctx dto_ctx;
typedef struct dto_pair dto_pair;

/* One task's optimum: OptimizationResultRecord (src/dto/results_objects.rs:14-24),
 * plus the grid indices of the chosen cell. */
typedef struct {
    uint32_t rank1;              /* threshold of list 1 */
    uint32_t rank2;              /* threshold of list 2 */
    int64_t set1_len;            /* #{rank1 <= threshold1} */
    int64_t set2_len;            /* #{rank2 <= threshold2} */
    int64_t population_size;
    int64_t intersection_size;
    double pvalue;               /* P(X >= k), X ~ Hypergeometric(N, set1_len, set2_len) */
    int32_t permuted;            /* 0 for the unpermuted task */
    int32_t i, j;                /* grid indices of (rank1, rank2) */
    int32_t status;              /* 0, or DTO_ERR_* for this task */
    int32_t route;               /* DTO_ROUTE_*: the search path that settled the task */
    int32_t reserved;
} dto_result;

/* Summary of a permutation run: the inputs of empirical_pvalue()
 * (src/stat_operations/empirical_pvalue.rs:109-187). */
typedef struct {
    int64_t n_perm;
    int64_t count_le;              /* #{permutation min-p <= unpermuted p} */
    double empirical_pvalue;       /* count_le / n_perm, or 1.0 when n_perm == 0 */
    double fdr;                    /* fdr(set1_len, set2_len, overlap, N, 0.8) */
    double logp_err_bound_screen;  /* |error| bound of the screen's log-pmf, in nats */
    double logp_err_bound_fp64;    /* relative error bound of an FP64 p-value */
    int64_t n_fallback;            /* tasks re-run by a slower exact path */
    int64_t n_refined;             /* FP64 tail evaluations */
    int64_t n_stage2;              /* FP32 tail evaluations of screened cells */
    double device_ms;              /* CUDA-event time of the device work */
    double grid_ms;                /* CUDA-event time of the grid (search) kernels */
    double perm_ms;                /* CUDA-event time of the permutation kernels */
    int64_t n_launches;            /* kernels launched */
    int64_t h2d_bytes;             /* host-to-device bytes copied by this call */
    int64_t d2h_bytes;             /* device-to-host bytes copied by this call */
    double sweep0_ms;              /* CUDA-event time of the table sweeps (levels 0-2 cascaded;
                                      main stream) */
    int64_t sweep0_launches;       /* their launches */
    int64_t sweep0_tasks;          /* permutations they took */
    int64_t n_route[DTO_ROUTES];   /* tasks (unpermuted included) settled by each DTO_ROUTE_* */
    double tail_ms;                /* device time from the end of the last table sweep to the end
                                      of the run (0 when no table sweep ran) */
} dto_summary;

DTO_API int dto_version(void);
DTO_API const char* dto_status_string(int status);

/* Context: one CUDA device, one stream, the device-resident log-factorial
 * tables and the per-batch scratch.  Replaces the thread pool and shared state
 * of run_single_node (src/run/single_node.rs:83-137). */
DTO_API int dto_ctx_create(int device, dto_ctx** out);
DTO_API int dto_ctx_destroy(dto_ctx* ctx);
DTO_API const char* dto_last_error(const dto_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * work around the library's launches. */
DTO_API void* dto_ctx_stream(dto_ctx* ctx);

/* RankedFeatureList::generate_thresholds (src/collections/ranked.rs:359-375),
 * including its quirk: the last threshold is not clamped to max_rank.
 * Writes min(count, cap) thresholds; returns count. */
DTO_API int64_t dto_generate_thresholds(uint32_t max_rank, uint32_t* out, int64_t cap);

/* The stable order by rank that dto_pair_create uses for each list
 * (src/collections/ranked.rs:527-542, a stable sort by rank): order[k] is the
 * input index of the k-th feature, equal ranks in input order.  Host only. */
DTO_API int dto_rank_order(const uint32_t* ranks, int64_t n, int32_t* order);

/* A list pair, resident on the device.  Replaces RankedFeatureList::from for
 * both lists (src/collections/ranked.rs:176-191: stable sort by rank, then the
 * thresholds) and the per-task set extraction (ranked.rs:561-568).
 *   ranks*, feat*: per input feature, in input order.  feat ids are unique in a
 *   list and lie in [0, n_features).
 *   population:   N of the hypergeometric (compute_population_size,
 *                 src/dto/compute_population_size.rs:66-104, done by the caller).
 * Errors: empty lists or no thresholds, duplicate or out-of-range ids,
 * population smaller than a list -> DTO_ERR_INVALID. */
DTO_API int dto_pair_create(dto_ctx* ctx, const uint32_t* ranks1, const int32_t* feat1, int64_t n1,
                    const uint32_t* ranks2, const int32_t* feat2, int64_t n2,
                    int64_t n_features, int64_t population, dto_pair** out);
DTO_API int dto_pair_destroy(dto_pair* pair);
/* Grid shape and the sorted order: order*[position] = input index. Any output
 * pointer may be NULL. */
DTO_API int dto_pair_info(const dto_pair* pair, int64_t* n_thresholds1, int64_t* n_thresholds2,
                  int64_t* n_common);
DTO_API int dto_pair_thresholds(const dto_pair* pair, uint32_t* t1, uint32_t* t2);
/* Philox stream id of the pair's permutations (default 0): permutation t of a
 * pair is a function of (seed, stream id, t).  Pairs that share a seed get
 * independent permutations by taking different stream ids. */
DTO_API int dto_pair_set_stream(dto_pair* pair, uint32_t stream_id);
/* No counterpart in the reference.  The pair's table ladder (the bounds that
 * decide which table screen settles each permutation of a long run) from a
 * sample of minimum p-values, e.g. a previous run's out_minp saved by another
 * process; count = 0 forgets the pair's ladder, so that its next long run
 * starts from the context's ladder for the pair's shape (that of the last
 * pair of that shape the context ran, within 5 % in every size) or, if there
 * is none, measures it from a first batch.  The ladder decides only which
 * path settles a task, never a result.  p-values outside [0, 1] ->
 * DTO_ERR_INVALID. */
DTO_API int dto_pair_set_ladder(dto_pair* pair, const double* minp, int64_t count);
/* No counterpart in the reference.  The quantile of the minimum p-values that
 * sets the pair's level-0 table (default 0.85; [0.5, 0.99], else
 * DTO_ERR_INVALID).  A pair with a ladder rebuilds it from its last run's
 * sample at the new quantile.  Performance only: results do not change. */
DTO_API int dto_pair_set_level0_quantile(dto_pair* pair, double q0);
/* No counterpart in the reference.  Tunes the pair's level-0 quantile by
 * timed trials: one run of n_perm permutations (> 1,024), then three runs per
 * candidate quantile (0.80, 0.85, 0.90), all of the same permutations, each
 * candidate's fastest device time of its last two counted (its first rebuilds
 * the table screens); the fastest candidate stays set on the pair and is
 * recorded for its shape, so that later pairs of that shape (within 5 % in
 * every size) start with it.  The trial runs' results are discarded. */
DTO_API int dto_pair_tune(dto_ctx* ctx, dto_pair* pair, int64_t n_perm, uint64_t seed, double* best_quantile);
/* Host-to-device bytes that dto_pair_create copied (the pair's device tables). */
DTO_API int64_t dto_pair_upload_bytes(const dto_pair* pair);
DTO_API int dto_pair_order(const dto_pair* pair, int32_t* order1, int32_t* order2);

/* The permutation null: the unpermuted task plus n_perm permuted tasks
 * (src/main.rs:122-126, src/run/single_node.rs:83-137), all on the device.
 *   seed:      Philox4x32-10 key of the on-device permutations; task t >= 1 uses
 *              permutation id t.
 *   perm_idx:  NULL, or the permuted views' index arrays to use instead
 *              (src/collections/permuted.rs:34), host memory laid out
 *              [n_perm][n1 + n2]: idx1 (positions of list 1) then idx2.
 *   out_unpermuted: the unpermuted optimum (NULL: not run, see dto_run_range).
 *   out_minp:  NULL or [n_perm] per-permutation minimum p-values.
 *   out_perm:  NULL or [n_perm] per-permutation optima.
 *   out_summary: NULL or the empirical p-value, FDR and error bounds.
 * Search path (never the results): a screen run of more than 1,024
 * permutations, or of at least 256 for a pair with a ladder of its own, goes
 * through the table ladder; other runs through the exhaustive screen.  A
 * screen run of at least 256 permutations leaves the pair its ladder. */
DTO_API int dto_run(dto_ctx* ctx, dto_pair* pair, int64_t n_perm, uint64_t seed, const int32_t* perm_idx,
            int precision, dto_result* out_unpermuted, double* out_minp, dto_result* out_perm,
            dto_summary* out_summary);

/* dto_run over permutation ids perm_first .. perm_first + n_perm - 1 (dto_run
 * is perm_first = 1).  A permutation depends only on (seed, pair, id), so
 * processes that split an id range between them (one GPU each) reproduce a
 * single run exactly; this replaces the MPI scatter of task chunks in
 * run_multi_node (src/run/multi_node.rs:114-161).  out_unpermuted may be NULL
 * here: the unpermuted task is then not run (replicas other than the one that
 * computes the observed optimum), and the summary's count_le is -1 and its
 * empirical_pvalue and fdr NaN. */
DTO_API int dto_run_range(dto_ctx* ctx, dto_pair* pair, uint32_t perm_first, int64_t n_perm,
                          uint64_t seed, const int32_t* perm_idx, int precision,
                          dto_result* out_unpermuted, double* out_minp, dto_result* out_perm,
                          dto_summary* out_summary);

/* No counterpart in the reference.  dto_run_range for callers that cannot
 * allocate device memory when they run it: a process whose memory manager owns
 * every device allocation (a framework's fixed-budget pool, a host application
 * that hands out device memory itself), or a runtime that forbids allocation
 * on its request path.  It calls no allocating routine: permutation labels,
 * the task counter and the per-task optima live in a fixed 32 MiB device array
 * inside libdto.so (held on every GPU that loads the library until the process
 * exits).  The caller passes the pair (created beforehand with
 * dto_pair_create) and d_minp, device memory of n_perm doubles that receives
 * each permutation's minimum p-value (the same values as dto_run_range,
 * exhaustive screen).  At most
 * 32 MiB / (24 + 2 * round8(n1) [+ 4 (n1 + n2) when the lists' feature sets
 * differ]) permutations per call (about 830 at n1 = n2 = 20,000); larger
 * n_perm -> DTO_ERR_INVALID.  The work is enqueued on the context's stream and
 * the call returns without waiting.  The first call on a device resolves the
 * array's device address (in the device's primary context) and should come
 * before any stream capture.  Calls share the array: calls whose GPU work
 * overlaps race. */
DTO_API int dto_run_range_noalloc(dto_ctx* ctx, dto_pair* pair, uint32_t perm_first, int64_t n_perm,
                                  uint64_t seed, double* d_minp);

/* One task: optimize(list1, list2, permute, population, debug=false)
 * (src/dto/optimize_main.rs:53-118).  permute != 0 uses permutation perm_id of
 * seed, or idx1/idx2 when both are non-NULL. */
DTO_API int dto_optimize(dto_ctx* ctx, dto_pair* pair, int permute, uint64_t seed, uint32_t perm_id,
                 const int32_t* idx1, const int32_t* idx2, int precision, dto_result* out);

/* OptimizationResult::Debug (src/dto/optimize_main.rs:68-70,
 * src/dto/process_threshold_pairs.rs:111-127): every cell's record, in the
 * reference's order (threshold1 major).  records holds n_thresholds1 *
 * n_thresholds2 entries. idx1/idx2 as in dto_optimize (NULL: unpermuted). */
DTO_API int dto_grid_dump(dto_ctx* ctx, dto_pair* pair, const int32_t* idx1, const int32_t* idx2,
                  dto_result* records);

/* hypergeometric_pvalue (src/stat_operations/hypergeometric_pvalue.rs:33-50)
 * for count quadruples, evaluated on the device with the engine's FP64 tail.
 * K > N or n > N -> DTO_ERR_INVALID (the reference panics). */
DTO_API int dto_hypergeom_sf(dto_ctx* ctx, const int64_t* N, const int64_t* K, const int64_t* n,
                     const int64_t* k, double* out, int64_t count);

/* The on-device permutations of tasks perm_first .. perm_first+count-1 as the
 * reference's index arrays (permuted.rs:34), so that dto_run with perm_idx
 * reproduces them.  idx1: [count][n1], idx2: [count][n2]. */
DTO_API int dto_export_permutations(dto_ctx* ctx, dto_pair* pair, uint64_t seed, uint32_t perm_first,
                            int64_t count, int32_t* idx1, int32_t* idx2);

/* fdr (src/stat_operations/fdr.rs:29-60). */
DTO_API double dto_fdr(int64_t set1_len, int64_t set2_len, int64_t overlap, int64_t population,
               double sensitivity);

/* ---- Many pairs, many requests ----
 * The reference runs one permutation null per process (src/main.rs:122-166,
 * tasks over threads in src/run/single_node.rs:83-137); these entry points run
 * many at once on one GPU.  A server owns `lanes` lanes (streams, scratch and
 * table screens of their own) and one worker thread per lane.  Requests queue
 * in arrival order; the head is admitted when a lane is free and its device
 * working set (dto_run_device_bytes) fits under mem_budget bytes next to the
 * requests running (mem_budget 0: no budget; a request larger than the budget
 * runs alone).  A worker that admits a short screen request (1,025 to 32,767
 * permutations of lists over one feature set, with a ladder from an earlier
 * run of the pair or of a pair of its shape) also takes the queued requests
 * of that kind that fit, in arrival
 * order, and sweeps their tasks together in waves (one launch over several
 * pairs).  A request's results equal dto_run_range's for the same arguments,
 * whatever runs beside it. */
typedef struct dto_server dto_server;
typedef int64_t dto_job;

DTO_API int dto_serve_create(dto_ctx* ctx, int lanes, int64_t mem_budget, dto_server** out);
/* Waits for every queued and running request, then frees the server. */
DTO_API int dto_serve_destroy(dto_server* srv);
/* Queues dto_run_range(pair, perm_first, n_perm, seed, precision) without a
 * test-mode index array.  The output buffers (out_minp: n_perm doubles,
 * nullable; out_summary nullable) must stay valid until the request is
 * waited for. */
DTO_API int dto_serve_submit(dto_server* srv, dto_pair* pair, uint32_t perm_first, int64_t n_perm,
                             uint64_t seed, int precision, dto_result* out_unpermuted, double* out_minp,
                             dto_summary* out_summary, dto_job* job);
/* *done = 1 once the request has finished (its outputs are written). */
DTO_API int dto_serve_poll(dto_server* srv, dto_job job, int* done);
/* Blocks until the request finishes, returns its status and forgets it;
 * queue_ms / run_ms (nullable) get the host wall time from submission to
 * admission and from admission to completion. */
DTO_API int dto_serve_wait(dto_server* srv, dto_job job, double* queue_ms, double* run_ms);
/* No counterpart in the reference (its tasks are joined without a limit,
 * src/run/single_node.rs:131-133).  dto_serve_wait with a limit: a request
 * not finished within timeout_ms returns DTO_ERR_TIMEOUT and stays known (wait
 * again, or cancel it). */
DTO_API int dto_serve_wait_for(dto_server* srv, dto_job job, double timeout_ms, double* queue_ms,
                               double* run_ms);
/* No counterpart in the reference.  Cancels a request: a queued one leaves the
 * queue at once, a running one stops at its next batch boundary once its
 * kernels in flight have finished (they are not interrupted).  Its wait then
 * returns DTO_ERR_CANCELLED and its outputs are undefined; a request that had
 * already finished, or that runs in a wave (which runs to its end), keeps its
 * results. */
DTO_API int dto_serve_cancel(dto_server* srv, dto_job job);
DTO_API const char* dto_serve_last_error(dto_server* srv);
DTO_API int dto_serve_stats(dto_server* srv, int64_t* queued, int64_t* running, int64_t* completed,
                            int64_t* reserved_bytes);
/* Device bytes a dto_run_range of n_perm permutations of the pair holds at
 * its peak (the admission size of a request). */
DTO_API int64_t dto_run_device_bytes(const dto_pair* pair, int64_t n_perm);
/* The permutation null of npairs pairs (pair q: n_perm[q] permutations from
 * id 1 of seeds[q]); per-pair outputs as in dto_run_range (out_minp[q] and
 * out_summary nullable).  Short screen runs of pairs with a ladder (as for a
 * server's waves) go in waves on the context's own stream: each wave draws
 * the labels of several pairs and sweeps all their tasks in one launch, and
 * each pair keeps the table screens built for it; the other runs go over
 * `lanes` lanes (<= 0: 4) meanwhile.  A wave's summary times are the wave's,
 * shared by its pairs in proportion to their tasks. */
DTO_API int dto_batch_run(dto_ctx* ctx, int npairs, dto_pair* const* pairs, const int64_t* n_perm,
                          const uint64_t* seeds, int precision, int lanes, dto_result* out_unpermuted,
                          double* const* out_minp, dto_summary* out_summary);

#ifdef __cplusplus
}
#endif

#endif /* DTO_H */
