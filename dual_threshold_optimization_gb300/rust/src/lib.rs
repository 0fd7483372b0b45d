//! The GB300 Dual Threshold Optimization engine from Rust: safe wrappers over
//! the C ABI of libdto (include/dto.h), shaped like the reference crate's
//! library surface so that its callers can switch:
//!
//! | here | reference |
//! |---|---|
//! | [`optimize`] | `optimize`, src/dto/optimize_main.rs:53-118 |
//! | [`run_single_node`] | `run_single_node`, src/run/single_node.rs:83-137 |
//! | [`hypergeometric_pvalue`] | src/stat_operations/hypergeometric_pvalue.rs:33-50 |
//! | [`empirical_pvalue`] | src/stat_operations/empirical_pvalue.rs:109-187 |
//! | [`fdr`] | src/stat_operations/fdr.rs:29-60 |
//!
//! The searches run on the GPU.  Like the reference, the free functions panic
//! with the library's message when a call fails; [`Engine`] and [`Pair`]
//! return `Result`s.  Permutation t of a run is permutation id t of a
//! counter-based Philox stream (the reference draws from an unseeded
//! thread_rng), so a fixed seed reproduces a run.
pub mod ffi;

use std::collections::HashMap;
use std::ffi::CStr;
use std::fmt;
use std::os::raw::c_int;
use std::sync::atomic::{AtomicU64, Ordering};
use std::sync::OnceLock;
use std::time::{SystemTime, UNIX_EPOCH};

/// A failed library call: its DTO_ERR_* status and message.
#[derive(Clone, Debug)]
pub struct Error {
    pub status: i32,
    pub message: String,
}

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "{} (status {})", self.message, self.status)
    }
}

impl std::error::Error for Error {}

pub type Result<T> = std::result::Result<T, Error>;

fn status_message(status: c_int) -> String {
    unsafe { CStr::from_ptr(ffi::dto_status_string(status)).to_string_lossy().into_owned() }
}

/// A ranked feature list: feature ids and their ranks, in any order (the
/// engine sorts stably by rank, src/collections/ranked.rs:527-542).
#[derive(Clone, Debug)]
pub struct RankedFeatureList {
    pub features: Vec<String>,
    pub ranks: Vec<u32>,
}

impl RankedFeatureList {
    pub fn from(features: Vec<String>, ranks: Vec<u32>) -> Result<Self> {
        if features.len() != ranks.len() {
            return Err(Error { status: ffi::DTO_ERR_INVALID, message: "features and ranks differ in length".into() });
        }
        Ok(RankedFeatureList { features, ranks })
    }

    pub fn len(&self) -> usize {
        self.features.len()
    }

    pub fn is_empty(&self) -> bool {
        self.features.is_empty()
    }
}

/// One task's optimum (src/dto/results_objects.rs:14-24).
#[derive(Clone, Debug, PartialEq)]
pub struct OptimizationResultRecord {
    pub rank1: u32,
    pub rank2: u32,
    pub set1_len: usize,
    pub set2_len: usize,
    pub population_size: u64,
    pub intersection_size: usize,
    pub pvalue: f64,
    pub permuted: bool,
}

impl From<&ffi::dto_result> for OptimizationResultRecord {
    fn from(r: &ffi::dto_result) -> Self {
        OptimizationResultRecord {
            rank1: r.rank1,
            rank2: r.rank2,
            set1_len: r.set1_len as usize,
            set2_len: r.set2_len as usize,
            population_size: r.population_size as u64,
            intersection_size: r.intersection_size as usize,
            pvalue: r.pvalue,
            permuted: r.permuted != 0,
        }
    }
}

/// OptimizationResult::Best or ::Debug (src/dto/results_objects.rs:26-32);
/// Debug holds every cell's record, threshold 1 major.
#[derive(Clone, Debug, PartialEq)]
pub enum OptimizationResult {
    Best(OptimizationResultRecord),
    Debug(Vec<OptimizationResultRecord>),
}

/// src/run/task.rs:3-9: task 0 is the unpermuted pair, tasks 1..=P permuted.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub struct Task {
    pub id: usize,
    pub permute: bool,
}

/// The tasks of src/main.rs:122-126.
pub fn make_tasks(permutations: usize) -> Vec<Task> {
    (0..=permutations).map(|id| Task { id, permute: id > 0 }).collect()
}

/// Precision of the threshold-pair search.
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    /// Plain FP64 tail of every cell.
    Fp64,
    /// 32-bit log-space screen, FP64 refine of the cells within the proven
    /// margin: the same optimum and p-value as Fp64.
    Screen,
}

impl Precision {
    fn code(self) -> c_int {
        match self {
            Precision::Fp64 => ffi::DTO_PRECISION_FP64,
            Precision::Screen => ffi::DTO_PRECISION_SCREEN,
        }
    }
}

/// One CUDA device: streams, log-factorial tables, scratch (dto_ctx).
pub struct Engine {
    ctx: *mut ffi::dto_ctx,
}

// The library serialises the context-level calls under the context's mutex.
unsafe impl Send for Engine {}
unsafe impl Sync for Engine {}

impl Engine {
    pub fn new(device: i32) -> Result<Engine> {
        let mut ctx = std::ptr::null_mut();
        let st = unsafe { ffi::dto_ctx_create(device, &mut ctx) };
        if st != ffi::DTO_OK {
            return Err(Error { status: st, message: status_message(st) });
        }
        Ok(Engine { ctx })
    }

    fn check(&self, st: c_int) -> Result<()> {
        if st == ffi::DTO_OK {
            return Ok(());
        }
        let msg = unsafe { CStr::from_ptr(ffi::dto_last_error(self.ctx)).to_string_lossy().into_owned() };
        Err(Error { status: st, message: if msg.is_empty() { status_message(st) } else { msg } })
    }

    /// Both lists on the device.  Feature ids are mapped to dense integers
    /// shared by the two lists.
    pub fn pair(&self, list1: &RankedFeatureList, list2: &RankedFeatureList, population_size: usize) -> Result<Pair<'_>> {
        let mut ids: HashMap<&str, i32> = HashMap::new();
        let mut f1: Vec<i32> = Vec::with_capacity(list1.len());
        for f in &list1.features {
            let next = ids.len() as i32;
            f1.push(*ids.entry(f.as_str()).or_insert(next));
        }
        let mut f2: Vec<i32> = Vec::with_capacity(list2.len());
        for f in &list2.features {
            let next = ids.len() as i32;
            f2.push(*ids.entry(f.as_str()).or_insert(next));
        }
        let n_features = ids.len() as i64;
        let mut p = std::ptr::null_mut();
        let st = unsafe {
            ffi::dto_pair_create(self.ctx, list1.ranks.as_ptr(), f1.as_ptr(), f1.len() as i64, list2.ranks.as_ptr(),
                                 f2.as_ptr(), f2.len() as i64, n_features, population_size as i64, &mut p)
        };
        self.check(st)?;
        let (mut n1, mut n2) = (0i64, 0i64);
        unsafe { ffi::dto_pair_info(p, &mut n1, &mut n2, std::ptr::null_mut()) };
        Ok(Pair { eng: self, ptr: p, thresholds1: n1 as usize, thresholds2: n2 as usize })
    }

    /// P(X >= k), X ~ Hypergeometric(N, K, n), on the device.
    pub fn hypergeometric_pvalue(&self, population: u64, successes: u64, draws: u64, observed: u64) -> Result<f64> {
        let (a, b, c, d) = (population as i64, successes as i64, draws as i64, observed as i64);
        let mut out = 0f64;
        self.check(unsafe { ffi::dto_hypergeom_sf(self.ctx, &a, &b, &c, &d, &mut out, 1) })?;
        Ok(out)
    }
}

impl Drop for Engine {
    fn drop(&mut self) {
        unsafe { ffi::dto_ctx_destroy(self.ctx) };
    }
}

/// The process-wide engine of the free functions (device DTO_DEVICE, else 0).
pub fn default_engine() -> &'static Engine {
    static ENGINE: OnceLock<Engine> = OnceLock::new();
    ENGINE.get_or_init(|| {
        let dev = std::env::var("DTO_DEVICE").ok().and_then(|v| v.parse().ok()).unwrap_or(0);
        Engine::new(dev).expect("failed to open the GPU engine")
    })
}

/// The result of a permutation run.
#[derive(Clone, Debug)]
pub struct Run {
    pub unpermuted: OptimizationResultRecord,
    /// Per-permutation minimum p-values, permutation ids first.. in order.
    pub minp: Vec<f64>,
    /// Per-permutation optima (when asked for).
    pub permuted: Vec<OptimizationResultRecord>,
    pub summary: ffi::dto_summary,
}

/// A list pair resident on the device (dto_pair).
pub struct Pair<'e> {
    eng: &'e Engine,
    ptr: *mut ffi::dto_pair,
    pub thresholds1: usize,
    pub thresholds2: usize,
}

impl<'e> Pair<'e> {
    /// The unpermuted task and permutations first..first + n_perm - 1 of `seed`.
    pub fn run_range(&self, first: u32, n_perm: usize, seed: u64, precision: Precision, records: bool) -> Result<Run> {
        let mut unp = ffi::dto_result::default();
        let mut minp = vec![0f64; n_perm];
        let mut recs = if records { vec![ffi::dto_result::default(); n_perm] } else { Vec::new() };
        let mut summary = ffi::dto_summary::default();
        let st = unsafe {
            ffi::dto_run_range(self.eng.ctx, self.ptr, first, n_perm as i64, seed, std::ptr::null(), precision.code(),
                               &mut unp, minp.as_mut_ptr(),
                               if records { recs.as_mut_ptr() } else { std::ptr::null_mut() }, &mut summary)
        };
        self.eng.check(st)?;
        Ok(Run {
            unpermuted: OptimizationResultRecord::from(&unp),
            minp,
            permuted: recs.iter().map(OptimizationResultRecord::from).collect(),
            summary,
        })
    }

    /// dto_run: permutations 1..=n_perm.
    pub fn run(&self, n_perm: usize, seed: u64, precision: Precision, records: bool) -> Result<Run> {
        self.run_range(1, n_perm, seed, precision, records)
    }

    /// One task: the unpermuted pair, or permutation `perm_id` of `seed`.
    pub fn optimize(&self, permute: bool, seed: u64, perm_id: u32, precision: Precision) -> Result<OptimizationResultRecord> {
        let mut out = ffi::dto_result::default();
        let st = unsafe {
            ffi::dto_optimize(self.eng.ctx, self.ptr, permute as c_int, seed, perm_id, std::ptr::null(),
                              std::ptr::null(), precision.code(), &mut out)
        };
        self.eng.check(st)?;
        Ok(OptimizationResultRecord::from(&out))
    }

    /// The level-0 table's quantile of this pair (default 0.85, in [0.5, 0.99]);
    /// performance only.
    pub fn set_level0_quantile(&self, q0: f64) -> Result<()> {
        let st = unsafe { ffi::dto_pair_set_level0_quantile(self.ptr, q0) };
        self.eng.check(st)
    }

    /// dto_pair_tune: picks the level-0 quantile by timed trial runs of
    /// `n_perm` permutations (> 1,024) among 0.80, 0.85 and 0.90, keeps the
    /// fastest for this pair and records it for its shape; returns it.
    pub fn tune(&self, n_perm: usize, seed: u64) -> Result<f64> {
        let mut best = 0f64;
        let st = unsafe { ffi::dto_pair_tune(self.eng.ctx, self.ptr, n_perm as i64, seed, &mut best) };
        self.eng.check(st)?;
        Ok(best)
    }

    /// Every cell's record of the unpermuted task (OptimizationResult::Debug).
    pub fn grid_dump(&self) -> Result<Vec<OptimizationResultRecord>> {
        let mut recs = vec![ffi::dto_result::default(); self.thresholds1 * self.thresholds2];
        let st = unsafe {
            ffi::dto_grid_dump(self.eng.ctx, self.ptr, std::ptr::null(), std::ptr::null(), recs.as_mut_ptr())
        };
        self.eng.check(st)?;
        Ok(recs.iter().map(OptimizationResultRecord::from).collect())
    }
}

impl Drop for Pair<'_> {
    fn drop(&mut self) {
        unsafe { ffi::dto_pair_destroy(self.ptr) };
    }
}

fn fresh_seed() -> u64 {
    static COUNTER: AtomicU64 = AtomicU64::new(0);
    let t = SystemTime::now().duration_since(UNIX_EPOCH).map(|d| d.as_nanos() as u64).unwrap_or(0);
    t ^ COUNTER.fetch_add(1, Ordering::Relaxed).wrapping_mul(0x9E37_79B9_7F4A_7C15)
}

/// src/dto/optimize_main.rs:53-118: the threshold pair with the smallest
/// upper-tail hypergeometric p-value (ties: larger overlap, then smaller
/// (rank1, rank2)); `permute` shuffles both lists; `debug` returns every
/// cell's record (of the unpermuted lists).
pub fn optimize(list1: &RankedFeatureList, list2: &RankedFeatureList, permute: bool, population_size: usize,
                debug: bool) -> OptimizationResult {
    let eng = default_engine();
    let pair = eng.pair(list1, list2, population_size).unwrap_or_else(|e| panic!("{}", e.message));
    if debug {
        return OptimizationResult::Debug(pair.grid_dump().unwrap_or_else(|e| panic!("{}", e.message)));
    }
    let rec = pair
        .optimize(permute, fresh_seed(), 1, Precision::Screen)
        .unwrap_or_else(|e| panic!("{}", e.message));
    OptimizationResult::Best(rec)
}

/// src/run/single_node.rs:83-137: every task, in task order.  All permuted
/// tasks run in one GPU call (num_threads is accepted and unused).
pub fn run_single_node(tasks: Vec<Task>, list1: RankedFeatureList, list2: RankedFeatureList, population_size: usize,
                       _num_threads: usize) -> Vec<OptimizationResult> {
    let eng = default_engine();
    let pair = eng.pair(&list1, &list2, population_size).unwrap_or_else(|e| panic!("{}", e.message));
    let max_id = tasks.iter().filter(|t| t.permute).map(|t| t.id).max().unwrap_or(0);
    let run = pair
        .run(max_id, fresh_seed(), Precision::Screen, true)
        .unwrap_or_else(|e| panic!("{}", e.message));
    tasks
        .iter()
        .map(|t| {
            if t.permute {
                assert!(t.id >= 1, "permuted task ids start at 1");
                OptimizationResult::Best(run.permuted[t.id - 1].clone())
            } else {
                OptimizationResult::Best(run.unpermuted.clone())
            }
        })
        .collect()
}

/// src/stat_operations/hypergeometric_pvalue.rs:33-50 on the device.
pub fn hypergeometric_pvalue(population: u64, successes: u64, draws: u64, observed: u64) -> f64 {
    default_engine()
        .hypergeometric_pvalue(population, successes, draws, observed)
        .unwrap_or_else(|_| panic!("Failed to create hypergeometric distribution"))
}

/// src/stat_operations/fdr.rs:29-60.
pub fn fdr(list1_len: usize, list2_len: usize, overlap: usize, population: usize, sensitivity: f64) -> f64 {
    assert!(sensitivity > 0.0, "Sensitivity must be greater than 0.");
    unsafe { ffi::dto_fdr(list1_len as i64, list2_len as i64, overlap as i64, population as i64, sensitivity) }
}

/// The output of src/stat_operations/empirical_pvalue.rs:109-187.
#[derive(Clone, Debug, PartialEq)]
pub struct EmpiricalPvalue {
    pub rank1: u32,
    pub rank2: u32,
    pub set1_len: usize,
    pub set2_len: usize,
    pub population_size: u64,
    pub unpermuted_intersection_size: usize,
    pub unpermuted_pvalue: f64,
    pub empirical_pvalue: f64,
    pub fdr: f64,
}

impl EmpiricalPvalue {
    /// Pretty JSON with the keys in sorted order, as the reference prints its
    /// serde_json map (src/main.rs:165).
    pub fn to_json_pretty(&self) -> String {
        format!(
            "{{\n  \"empirical_pvalue\": {:?},\n  \"fdr\": {:?},\n  \"population_size\": {},\n  \"rank1\": {},\n  \
             \"rank2\": {},\n  \"set1_len\": {},\n  \"set2_len\": {},\n  \"unpermuted_intersection_size\": {},\n  \
             \"unpermuted_pvalue\": {:?}\n}}",
            self.empirical_pvalue, self.fdr, self.population_size, self.rank1, self.rank2, self.set1_len,
            self.set2_len, self.unpermuted_intersection_size, self.unpermuted_pvalue
        )
    }
}

/// src/stat_operations/empirical_pvalue.rs:109-187: #{permuted p <= the
/// unpermuted p} / P (1.0 without permutations) and the FDR at sensitivity
/// 0.8.  Panics without an unpermuted result, as the reference does.
pub fn empirical_pvalue(results: &[OptimizationResult]) -> EmpiricalPvalue {
    let best: Vec<&OptimizationResultRecord> = results
        .iter()
        .filter_map(|r| if let OptimizationResult::Best(b) = r { Some(b) } else { None })
        .collect();
    let u = best.iter().find(|r| !r.permuted).expect("No unpermuted result found in the provided results.");
    let perm: Vec<f64> = best.iter().filter(|r| r.permuted).map(|r| r.pvalue).collect();
    let empirical = if perm.is_empty() {
        1.0
    } else {
        perm.iter().filter(|&&p| p <= u.pvalue).count() as f64 / perm.len() as f64
    };
    EmpiricalPvalue {
        rank1: u.rank1,
        rank2: u.rank2,
        set1_len: u.set1_len,
        set2_len: u.set2_len,
        population_size: u.population_size,
        unpermuted_intersection_size: u.intersection_size,
        unpermuted_pvalue: u.pvalue,
        empirical_pvalue: empirical,
        fdr: fdr(u.set1_len, u.set2_len, u.intersection_size, u.population_size as usize, 0.8),
    }
}

#[cfg(test)]
mod tests {
    // These run on a machine with a GB300 (the engine opens device 0).
    use super::*;

    fn test_data() -> (RankedFeatureList, RankedFeatureList) {
        // the 3 x 3 example of src/dto/process_threshold_pairs.rs:68
        let l1 = RankedFeatureList::from(vec!["gene1".into(), "gene2".into(), "gene3".into()], vec![1, 2, 3]).unwrap();
        let l2 = RankedFeatureList::from(vec!["gene1".into(), "gene2".into(), "gene3".into()], vec![1, 2, 3]).unwrap();
        (l1, l2)
    }

    #[test]
    fn debug_grid_has_nine_cells() {
        let (l1, l2) = test_data();
        match optimize(&l1, &l2, false, 3, true) {
            OptimizationResult::Debug(r) => assert_eq!(r.len(), 9),
            other => panic!("expected Debug, got {:?}", other),
        }
    }

    #[test]
    fn run_single_node_returns_every_task() {
        let (l1, l2) = test_data();
        let res = run_single_node(make_tasks(5), l1, l2, 3, 1);
        assert_eq!(res.len(), 6);
        let e = empirical_pvalue(&res);
        assert!(e.empirical_pvalue >= 0.0 && e.empirical_pvalue <= 1.0);
        assert!(e.to_json_pretty().starts_with("{\n  \"empirical_pvalue\": "));
    }
}
