//! Raw declarations of the C ABI in include/dto.h (libdto).  Every function
//! returns a status code (DTO_OK = 0); `dto_last_error` has the message.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const DTO_OK: c_int = 0;
pub const DTO_ERR_INVALID: c_int = 1;
pub const DTO_ERR_OOM: c_int = 2;
pub const DTO_ERR_TIMEOUT: c_int = 3;
pub const DTO_ERR_CUDA: c_int = 4;
pub const DTO_ERR_NOT_FOUND: c_int = 5;
pub const DTO_ERR_CANCELLED: c_int = 6;

pub const DTO_PRECISION_FP64: c_int = 0;
pub const DTO_PRECISION_SCREEN: c_int = 1;

pub const DTO_ROUTES: usize = 8;

#[repr(C)]
pub struct dto_ctx {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct dto_pair {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct dto_server {
    _opaque: [u8; 0],
}
pub type dto_job = i64;

/// One task's optimum (OptimizationResultRecord plus the grid indices).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct dto_result {
    pub rank1: u32,
    pub rank2: u32,
    pub set1_len: i64,
    pub set2_len: i64,
    pub population_size: i64,
    pub intersection_size: i64,
    pub pvalue: f64,
    pub permuted: i32,
    pub i: i32,
    pub j: i32,
    pub status: i32,
    pub route: i32,
    pub reserved: i32,
}

/// Summary of a permutation run.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dto_summary {
    pub n_perm: i64,
    pub count_le: i64,
    pub empirical_pvalue: f64,
    pub fdr: f64,
    pub logp_err_bound_screen: f64,
    pub logp_err_bound_fp64: f64,
    pub n_fallback: i64,
    pub n_refined: i64,
    pub n_stage2: i64,
    pub device_ms: f64,
    pub grid_ms: f64,
    pub perm_ms: f64,
    pub n_launches: i64,
    pub h2d_bytes: i64,
    pub d2h_bytes: i64,
    pub sweep0_ms: f64,
    pub sweep0_launches: i64,
    pub sweep0_tasks: i64,
    pub n_route: [i64; DTO_ROUTES],
    pub tail_ms: f64,
}

extern "C" {
    pub fn dto_version() -> c_int;
    pub fn dto_status_string(status: c_int) -> *const c_char;
    pub fn dto_ctx_create(device: c_int, out: *mut *mut dto_ctx) -> c_int;
    pub fn dto_ctx_destroy(ctx: *mut dto_ctx) -> c_int;
    pub fn dto_last_error(ctx: *const dto_ctx) -> *const c_char;
    pub fn dto_ctx_stream(ctx: *mut dto_ctx) -> *mut c_void;
    pub fn dto_generate_thresholds(max_rank: u32, out: *mut u32, cap: i64) -> i64;
    pub fn dto_rank_order(ranks: *const u32, n: i64, order: *mut i32) -> c_int;
    pub fn dto_pair_create(
        ctx: *mut dto_ctx,
        ranks1: *const u32,
        feat1: *const i32,
        n1: i64,
        ranks2: *const u32,
        feat2: *const i32,
        n2: i64,
        n_features: i64,
        population: i64,
        out: *mut *mut dto_pair,
    ) -> c_int;
    pub fn dto_pair_destroy(pair: *mut dto_pair) -> c_int;
    pub fn dto_pair_info(pair: *const dto_pair, n_thresholds1: *mut i64, n_thresholds2: *mut i64,
                         n_common: *mut i64) -> c_int;
    pub fn dto_pair_thresholds(pair: *const dto_pair, t1: *mut u32, t2: *mut u32) -> c_int;
    pub fn dto_pair_set_stream(pair: *mut dto_pair, stream_id: u32) -> c_int;
    pub fn dto_pair_set_ladder(pair: *mut dto_pair, minp: *const f64, count: i64) -> c_int;
    pub fn dto_pair_set_level0_quantile(pair: *mut dto_pair, q0: f64) -> c_int;
    pub fn dto_pair_tune(ctx: *mut dto_ctx, pair: *mut dto_pair, n_perm: i64, seed: u64, best_quantile: *mut f64)
        -> c_int;
    pub fn dto_pair_upload_bytes(pair: *const dto_pair) -> i64;
    pub fn dto_pair_order(pair: *const dto_pair, order1: *mut i32, order2: *mut i32) -> c_int;
    pub fn dto_run(
        ctx: *mut dto_ctx,
        pair: *mut dto_pair,
        n_perm: i64,
        seed: u64,
        perm_idx: *const i32,
        precision: c_int,
        out_unpermuted: *mut dto_result,
        out_minp: *mut f64,
        out_perm: *mut dto_result,
        out_summary: *mut dto_summary,
    ) -> c_int;
    pub fn dto_run_range(
        ctx: *mut dto_ctx,
        pair: *mut dto_pair,
        perm_first: u32,
        n_perm: i64,
        seed: u64,
        perm_idx: *const i32,
        precision: c_int,
        out_unpermuted: *mut dto_result,
        out_minp: *mut f64,
        out_perm: *mut dto_result,
        out_summary: *mut dto_summary,
    ) -> c_int;
    pub fn dto_run_range_noalloc(ctx: *mut dto_ctx, pair: *mut dto_pair, perm_first: u32, n_perm: i64,
                                 seed: u64, d_minp: *mut f64) -> c_int;
    pub fn dto_optimize(
        ctx: *mut dto_ctx,
        pair: *mut dto_pair,
        permute: c_int,
        seed: u64,
        perm_id: u32,
        idx1: *const i32,
        idx2: *const i32,
        precision: c_int,
        out: *mut dto_result,
    ) -> c_int;
    pub fn dto_grid_dump(ctx: *mut dto_ctx, pair: *mut dto_pair, idx1: *const i32, idx2: *const i32,
                         records: *mut dto_result) -> c_int;
    pub fn dto_hypergeom_sf(ctx: *mut dto_ctx, n_pop: *const i64, k_succ: *const i64, n_draw: *const i64,
                            k_obs: *const i64, out: *mut f64, count: i64) -> c_int;
    pub fn dto_export_permutations(ctx: *mut dto_ctx, pair: *mut dto_pair, seed: u64, perm_first: u32,
                                   count: i64, idx1: *mut i32, idx2: *mut i32) -> c_int;
    pub fn dto_fdr(set1_len: i64, set2_len: i64, overlap: i64, population: i64, sensitivity: f64) -> f64;
    pub fn dto_serve_create(ctx: *mut dto_ctx, lanes: c_int, mem_budget: i64, out: *mut *mut dto_server) -> c_int;
    pub fn dto_serve_destroy(srv: *mut dto_server) -> c_int;
    pub fn dto_serve_submit(
        srv: *mut dto_server,
        pair: *mut dto_pair,
        perm_first: u32,
        n_perm: i64,
        seed: u64,
        precision: c_int,
        out_unpermuted: *mut dto_result,
        out_minp: *mut f64,
        out_summary: *mut dto_summary,
        job: *mut dto_job,
    ) -> c_int;
    pub fn dto_serve_poll(srv: *mut dto_server, job: dto_job, done: *mut c_int) -> c_int;
    pub fn dto_serve_wait(srv: *mut dto_server, job: dto_job, queue_ms: *mut f64, run_ms: *mut f64) -> c_int;
    pub fn dto_serve_wait_for(srv: *mut dto_server, job: dto_job, timeout_ms: f64, queue_ms: *mut f64,
                              run_ms: *mut f64) -> c_int;
    pub fn dto_serve_cancel(srv: *mut dto_server, job: dto_job) -> c_int;
    pub fn dto_serve_last_error(srv: *mut dto_server) -> *const c_char;
    pub fn dto_serve_stats(srv: *mut dto_server, queued: *mut i64, running: *mut i64, completed: *mut i64,
                           reserved_bytes: *mut i64) -> c_int;
    pub fn dto_run_device_bytes(pair: *const dto_pair, n_perm: i64) -> i64;
    pub fn dto_batch_run(
        ctx: *mut dto_ctx,
        npairs: c_int,
        pairs: *const *mut dto_pair,
        n_perm: *const i64,
        seeds: *const u64,
        precision: c_int,
        lanes: c_int,
        out_unpermuted: *mut dto_result,
        out_minp: *const *mut f64,
        out_summary: *mut dto_summary,
    ) -> c_int;
}
