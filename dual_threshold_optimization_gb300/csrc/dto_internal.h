// dto_internal.h -- types shared by the kernels and the host side of libdto.so.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace dto {

constexpr int kGridWarps = 12;       // warps per CTA of the grid kernel (one task per warp)
constexpr int kCandCap = 64;         // per-warp candidate buffer of the screen
constexpr int kBucketBits = 12;
constexpr int kBuckets = 1 << kBucketBits;  // Rao-Sandelius buckets
static_assert(kBuckets % 1024 == 0, "perm_kernel: buckets must split evenly over its warps");
// Shared-memory budget of one permutation CTA (227 KB per block, less the
// static arrays).
constexpr size_t kPermSmemBudget = 226 * 1024;
__host__ __device__ constexpr size_t perm_round16(size_t b) { return (b + 15) & ~(size_t)15; }
// counters | indices; each region starts on a 16-byte boundary, the bucket /
// label area (L int16) follows where it fits
__host__ __device__ constexpr size_t perm_base_smem(int L) {
  return (size_t)kBuckets * 4 + perm_round16((size_t)L * 2);
}
__host__ __device__ constexpr bool perm_stage_area(int L) {
  return perm_base_smem(L) + perm_round16((size_t)L * 2) <= kPermSmemBudget;
}
constexpr int kMaxListLen = 65534;   // positions are uint16; overlaps stay below the 0xFFFF "never" mark
constexpr int kScreenSlack = 5;      // fixed-point units added to the screen threshold
constexpr int kSurvCap = 256;        // per-warp survivors of the FP32 stage

// Per-warp shared-memory layout of the grid kernel, in ints: the column
// counters (32 lanes x (C|1) slots, rounded to even), the candidate buffer
// (kCandCap int2) and the survivor list (cell, overlap, lo per entry).
__host__ __device__ constexpr int grid_cnt_ints(int C) { return (32 * (C | 1) + 1) & ~1; }
__host__ __device__ constexpr int grid_warp_ints(int C) { return grid_cnt_ints(C) + 2 * kCandCap + 3 * kSurvCap; }

// Device view of one list pair.  Rows are list-1 thresholds, columns list-2
// thresholds.  A "label" is the shared-memory slot of a list-2 threshold
// column in the grid kernel's per-warp counter array (column j of lane
// j / C lives at slot lane * (C|1) + j % C); -1 means the feature never
// enters a list-2 set (absent from list 2, or rank above the last threshold).
struct PairDev {
  int n1, n2;            // thresholds per list (grid rows, columns)
  int N1, N2;            // list lengths
  long long Npop;        // population size N of the hypergeometric
  int C;                 // columns per lane
  int fshift;            // fixed-point fraction bits of the screen table
  const int* rowstart;   // [n1+1]: list-1 positions of row i are [rowstart[i], rowstart[i+1])
  const int* ncnt;       // [n2]: set size of list 2 at threshold j
  const uint32_t* F;     // [Npop+1]: round(ln(m!) * 2^fshift) modulo 2^32
  const double2* LF;     // [>= Npop+1]: ln(m!) as double-double (hi, lo)
  const int16_t* Ylab;   // [N1]: label of the list-2 column of the feature at list-1 position p
  const int16_t* lab2;   // [N2]: label of list-2 position q
  const int* map12;      // [N1]: list-2 position of the feature at list-1 position p, or -1
};

// One task's optimum; route is the DTO_ROUTE_* code of the path that settled it.
struct TaskResult {
  double p;
  int i, j, k;
  int route;
};

enum GridMode { kModeFull64 = 0, kModeScreen = 1, kModeDump = 2 };

// The table sweep's per-lane layout (a half-warp's lane holds C2 = 2 C
// columns as C words of two 16-bit counts): columns padded to whole 16-byte
// chunks, and counter words per lane padded to an odd number of 16-byte
// chunks (a quarter-warp's 128-bit loads hit distinct banks).
__host__ __device__ constexpr int hw_cq(int C2) { return (C2 + 7) & ~7; }
__host__ __device__ constexpr int hw_wp(int C2) { return 4 * ((hw_cq(C2) / 8) | 1); }

// Column labels (the list-2 threshold column j of a list-1 position; -1:
// none) in two forms.  The grid kernel's: (j / C) * (C | 1) + j % C, its
// counter index (32 lanes of C columns, odd stride).  The table sweep's: the
// byte offset of the column's 16-bit count among the 16 lanes of a task
// (lane j / 2C, word (j % 2C) / 2), bit 13 set for the upper half of the
// word.  Labels drawn for the table sweep are in its form, so it adds them
// to its counters without a lookup; the grid kernel turns them back when it
// screens the tasks the sweep left.
__host__ __device__ constexpr int hw_label_of_column(int j, int C) {
  return (4 * ((j / (2 * C)) * hw_wp(2 * C) + (j % (2 * C)) / 2)) | ((j % 2) << 13);
}
__host__ __device__ constexpr int grid_label_of_column(int j, int C) { return (j / C) * (C | 1) + j % C; }
__host__ __device__ constexpr int column_of_hw_label(int v, int C) {
  return ((v & 0x1FFF) / 4 / hw_wp(2 * C)) * (2 * C) + 2 * (((v & 0x1FFF) / 4) % hw_wp(2 * C)) + ((v >> 13) & 1);
}

struct GridArgs {
  PairDev P;
  const int16_t* X;      // [ntask][xstride] labels per list-1 position
  long long xstride;
  int ntask;
  int mode;
  int route;             // DTO_ROUTE_* written with each result
  int smemF;             // 1: the fixed-point table is staged in shared memory
  int coop;              // screen mode: the CTA's warps share each task
  int hwlab;             // 1: X holds the table sweep's labels (a table run's fallbacks)
  TaskResult* out;       // [ntask]
  int* work;             // task counter (zeroed before the launch)
  unsigned long long* n_refined;  // [3]: FP64 tails, FP32 tails, speculative sweeps rejected
  unsigned* guess_hist;  // nullable: [257] histogram of finished tasks' bounds (screen mode)
  const int* task_list;  // nullable: task q is row/result task_list[q]
  const int* ntask_dev;  // nullable: the task count, read on the device
  int* dump_k;           // kModeDump: [n1*n2] overlaps
  double* dump_p;        // kModeDump: [n1*n2] p-values
};

struct PermArgs {
  int L;                 // list length
  uint64_t seed;
  uint32_t pair_id;
  uint32_t perm_base;    // permutation id of CTA 0
  uint32_t list_tag;     // 1 or 2
  const int16_t* Ylab;   // nullable: write labels X[p] = Ylab[sigma[p]]
  int16_t* X;
  long long xstride;
  int* sigma;            // nullable: write sigma [count][sstride]
  long long sstride;
  // With labels (X): the grid rows' position ranges, rowstart[0..n1].  Only
  // the multiset of labels inside each row reaches the search, so a bucket
  // whose positions lie inside one row keeps the order the scatter left
  // (nullable: every bucket shuffled as the specification says).
  const int* rowstart;
  int n1;
  // set by launch_perm: the bucket / label area fits in shared memory
  int stage;
};

struct ComposeArgs {
  int N1, N2;
  const int* idx1;       // row b at idx1 + b * stride, N1 entries
  const int* idx2;       // row b at idx2 + b * stride, N2 entries, or nullptr (identity)
  long long stride;
  const int* map12;
  const int16_t* lab2;
  int16_t* X;
  long long xstride;
};

// Table screen (dto_table.cuh).
// Warps per CTA of the table-screen kernel and the CTAs per SM its register
// budget is compiled for.  One CTA of 16 warps per SM gives each thread 128
// registers, which keeps the row sweep free of register spills; at 2 CTAs
// (64 registers) spilled state reloads from L2 inside the sweep and the
// kernel runs about 25 % slower.
constexpr int kTableWarps = 16;
constexpr int kTableCtasPerSm = 1;
constexpr int kTableHitCap = 8192;  // hit slots per task
// hit slots per warp of a table sweep (the half-warp sweep runs two tasks)
constexpr int kTableWarpHits = 2 * kTableHitCap;


struct TableArgs {
  int n1, n2, N, C;      // C: columns per lane of the half-warp sweep (2 C of the pair)
  const int* rowstart;   // K_i = rowstart[i+1]
  const int* ncnt;
  // m_j = list-1 positions whose label is <= j (any permutation: the labels
  // are only moved), and N1 = all list-1 positions; a cell's overlap lies in
  // [max(0, K_i + m_j - N1), min(K_i, m_j)]
  const int* mcnt;
  int N1;
  const uint32_t* F;
  int fshift;
  int tau;               // fixed-point ln p guess
  uint16_t* kthr;        // [n1][table_cq(C) / 8][lanes][8]
};

struct TableGridArgs {
  PairDev P;
  const int16_t* X;
  long long xstride;
  int ntask;
  int tau;                // the guess the table was built for
  const uint16_t* kthr;   // table_build_kernel's layout for the sweep that reads it
  // tighter tables (bounds tight_tau[0] > tight_tau[1] > ...): once a
  // resolve has set a task's bound B, its remaining rows are swept against
  // the tightest table whose bound is still >= B
  const uint16_t* tight[3];
  int tight_tau[3];
  int ntight;
  // The half-warp sweep cascades: a task with no hit at level l is swept
  // again at level l + 1 by the same half-warp, up to nlev levels (the level
  // above sits in kthr, tau, tight*, ntight; levels 1 and 2 below).  Tasks
  // of the last level with no hit go to the fallback list.  nlev = 1: one
  // level.
  int nlev;
  const uint16_t* kthr_up[2];
  int tau_up[2];
  const uint16_t* tight_up[2][3];
  int tight_tau_up[2][3];
  int ntight_up[2];
  int route;              // DTO_ROUTE_* written with each result
  int smemF;              // the ln m! table is copied to shared memory
  TaskResult* out;
  int* work;
  unsigned long long* n_refined;  // [3]
  int* fallback;          // [ntask] task ids whose minimum lies above the guess
  int* nfallback;         // count (zeroed before the launch)
  const int* task_list;   // nullable: task q is row/result task_list[q]
  const int* ntask_dev;   // nullable: the task count, read on the device
  int2* hitbuf;           // [gridDim.x * kTableWarps][hitcap] hits (packed cell, overlap)
  int hitcap;
  // nullable: a cascade sweep over several packed pairs of the same C, one
  // TableGridArgs per pair (segment, in device memory); the launch's own
  // fields then give only C, hitbuf and hitcap
  const TableGridArgs* segs;
  int nseg;
};

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The limit only ever grows, so launches from several host
// threads (executor lanes) never see it lowered between their own set and
// launch.
cudaError_t raise_smem_limit(const void* kernel, size_t bytes);

size_t grid_smem_bytes(int C, int n1, long long Npop, int smemF);
// C is the pair's columns per lane of the 32-lane layout; the table sweep is
// the half-warp sweep (16 lanes of 2 C columns).
size_t table_smem_bytes(int C, int n1, int n2, long long Npop, int smemF);
size_t table_entries(int C, int n1);
cudaError_t launch_table_build(const TableArgs& a, int nsm, cudaStream_t s);
cudaError_t launch_table_grid(const TableGridArgs& a, int C, int ctas, cudaStream_t s);
cudaError_t launch_grid(const GridArgs& a, int grid_ctas, cudaStream_t s);
cudaError_t launch_perm(const PermArgs& a, int count, cudaStream_t s);
cudaError_t launch_compose(const ComposeArgs& a, int count, cudaStream_t s);
cudaError_t noalloc_scratch(int device, void** ptr, size_t* bytes);
cudaError_t launch_noalloc_copy_p(const TaskResult* r, double* out, int n, cudaStream_t s);
cudaError_t launch_sf_batch(const double2* LF, const long long* q, double* out, long long count,
                            cudaStream_t s);

// Per-C instantiations of the grid kernel (one translation unit each).
#define DTO_FOR_EACH_C(X) X(4) X(8) X(12) X(16) X(20) X(24) X(28) X(32)
#define DTO_DECLARE_GRID(CC) cudaError_t launch_grid_c##CC(const GridArgs& a, int ctas, size_t smem, cudaStream_t s);
DTO_FOR_EACH_C(DTO_DECLARE_GRID)
#undef DTO_DECLARE_GRID
#define DTO_DECLARE_TABLE(CC) cudaError_t launch_table_grid_c##CC(const TableGridArgs& a, int ctas, size_t smem, cudaStream_t s);
DTO_FOR_EACH_C(DTO_DECLARE_TABLE)
#undef DTO_DECLARE_TABLE

}  // namespace dto
