// dto_kernels.cu -- permutation, composition and tail kernels, and the grid
// kernel dispatcher.
//
// Permutations replace PermutedRankedFeatureList::new
// (src/collections/permuted.rs:56-60: a uniform shuffle of 0..len with
// rand's thread_rng).  Here a permutation is a deterministic function of
// (seed, pair id, permutation id, list tag):
//   1. element e draws a bucket in [0, 4096): the top 12 bits of the low
//      (e even) or high (e odd) 16-bit half of word (e/2) % 4 of the
//      Philox4x32-10 block at counter (e/8, perm, pair, 0x10000000 | tag<<24)
//      (key = the two halves of the seed): eight elements per block;
//   2. elements are grouped by bucket, in increasing element order inside a
//      bucket;
//   3. each bucket is shuffled by the forward Fisher-Yates pass (i = 1..sz-1:
//      swap positions i and j, j uniform in [0, i]), the draws taken from the
//      bucket's own Philox stream (counter (call, perm, pair,
//      0x20000000 | tag<<24 | bucket), the four words of each call in order)
//      by Lemire's multiply-shift with rejection.
// One level of Rao-Sandelius bucketing followed by uniform shuffles of the
// buckets gives an exactly uniform permutation.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "dto_grid.cuh"
#include "dto_internal.h"
#include "dto_table.cuh"
#include "dto_math.cuh"

namespace dto {

struct PhiloxStream {
  uint4 ctr;
  uint32_t k0, k1;
  uint4 buf;
  int used;
  __device__ __forceinline__ uint32_t next() {
    if (used == 4) {
      buf = philox4x32_10(ctr, k0, k1);
      ctr.x += 1;
      used = 0;
    }
    uint32_t w = (used == 0) ? buf.x : (used == 1) ? buf.y : (used == 2) ? buf.z : buf.w;
    ++used;
    return w;
  }
  __device__ __forceinline__ uint32_t bounded(uint32_t range) {
    uint32_t xw = next();
    unsigned long long m = (unsigned long long)xw * range;
    uint32_t l = (uint32_t)m;
    if (l < range) {
      uint32_t thr = (0u - range) % range;
      while (l < thr) {
        xw = next();
        m = (unsigned long long)xw * range;
        l = (uint32_t)m;
      }
    }
    return (uint32_t)(m >> 32);
  }
};

// One CTA per permutation.  Shared memory: the bucket counters (int32,
// kBuckets; after the scatter they hold each bucket's end), the shuffled
// element indices (uint16, L) and, where it fits, an area of L int16 that
// first holds each element's bucket (so that the scatter and the row starts
// need not redraw the Philox blocks) and then the staged label table.
// kBuckets = 4096 keeps buckets at a few elements for the list lengths of
// interest, so the per-bucket canonical sort and Fisher-Yates pass are a few
// operations per element.
template <int kPermThreads>
__device__ __forceinline__ void perm_body(const PermArgs& A, int* cnt, uint16_t* sA, int16_t* sY) {
  __shared__ int warpTot[kPermThreads / 32];
  __shared__ int nClaim;  // claimed buckets in the list (rows longer than the CTA)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int L = A.L;
  const uint32_t perm = A.perm_base + blockIdx.x;
  const uint32_t k0 = (uint32_t)A.seed, k1 = (uint32_t)(A.seed >> 32);
  const uint32_t tagB = 0x10000000u | (A.list_tag << 24);
  static_assert(kBucketBits == 12, "buckets are the top 12 bits of a 16-bit half");
  static_assert(4 * kPermThreads <= kBuckets, "the claim list (two ints a row start) fits in the counters");
  auto bucket_in = [](const uint4& w, int e) -> int {
    const int q = (e >> 1) & 3;
    const uint32_t word = q == 0 ? w.x : q == 1 ? w.y : q == 2 ? w.z : w.w;
    return (int)((e & 1) ? (word >> 20) : ((word >> 4) & 0xFFFu));
  };
  auto bucket_of = [&](int e) -> int {  // redrawn from its Philox block
    return bucket_in(philox4x32_10(make_uint4((uint32_t)(e >> 3), perm, A.pair_id, tagB), k0, k1), e);
  };

  for (int b = tid; b < kBuckets; b += kPermThreads) cnt[b] = 0;
  const bool rows = A.X && A.rowstart;
  // The label table goes to shared memory by asynchronous 16-byte copies
  // (waited for before the gather).  The label area first holds each
  // element's bucket (uint16), so that the scatter need not redraw the
  // blocks; the copies start once the row starts have found their buckets,
  // and land during the shuffles.  (Up to two row starts a thread: longer
  // grids redraw.)
  const bool asyncY = sY && (reinterpret_cast<uintptr_t>(A.Ylab) & 15) == 0;
  const bool ids = sY && (!rows || A.n1 + 1 <= 2 * kPermThreads);
  uint16_t* sId = reinterpret_cast<uint16_t*>(sY);
  auto stage_labels = [&]() {
    if (!A.X) return;
    if (asyncY) {
      const char* src = reinterpret_cast<const char*>(A.Ylab);
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sY);
      const int bytes = 2 * L;
      for (int o = 16 * tid; o < bytes; o += 16 * kPermThreads) {
        const int n = min(16, bytes - o);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst + o), "l"(src + o), "r"(n)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    } else if (sY) {
      for (int q = tid; q < L; q += kPermThreads) sY[q] = __ldg(A.Ylab + q);
    }
  };
  if (!ids) stage_labels();
  // this thread's first two row starts (and the ones before them), loaded
  // now so that the loads are done by the time the shuffles need them
  const int r1 = tid + kPermThreads;
  const int rsPrev0 = (rows && tid >= 1 && tid <= A.n1) ? __ldg(A.rowstart + tid - 1) : 0;
  const int rs0 = (rows && tid <= A.n1) ? __ldg(A.rowstart + tid) : 0;
  const int rsPrev1 = (rows && r1 <= A.n1) ? __ldg(A.rowstart + r1 - 1) : 0;
  const int rs1 = (rows && r1 <= A.n1) ? __ldg(A.rowstart + r1) : 0;
  __syncthreads();
  // counting: one Philox block per eight elements; their eight buckets go to
  // the bucket area as one 16-byte store (the area is a whole number of
  // 16-byte chunks, so the padding past L takes the last group's spare ids)
  const int groups = (L + 7) >> 3;
  for (int g = tid; g < groups; g += kPermThreads) {
    const uint4 w = philox4x32_10(make_uint4((uint32_t)g, perm, A.pair_id, tagB), k0, k1);
    const uint32_t wv[4] = {w.x, w.y, w.z, w.w};
    uint32_t packed[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) packed[q] = ((wv[q] >> 4) & 0xFFFu) | ((wv[q] >> 20) << 16);
    if (ids) reinterpret_cast<uint4*>(sId)[g] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = 8 * g + q;
      if (e < L) atomicAdd(&cnt[(int)((q & 1) ? (wv[q >> 1] >> 20) : ((wv[q >> 1] >> 4) & 0xFFFu))], 1);
    }
  }
  __syncthreads();
  // exclusive scan of the counters: thread t holds kPerThread consecutive
  // counters (a serial prefix), one warp scan of the threads' totals, one of
  // the warps' totals
  {
    constexpr int kPerThread = kBuckets / kPermThreads;
    static_assert(kPerThread % 4 == 0, "counters a thread: whole int4");
    int4* c4 = reinterpret_cast<int4*>(cnt) + tid * (kPerThread / 4);
    int v[kPerThread];
#pragma unroll
    for (int k = 0; k < kPerThread / 4; ++k) {
      const int4 x = c4[k];
      v[4 * k] = x.x;
      v[4 * k + 1] = x.y;
      v[4 * k + 2] = x.z;
      v[4 * k + 3] = x.w;
    }
    int tot = 0;
#pragma unroll
    for (int k = 0; k < kPerThread; ++k) {
      const int x = v[k];
      v[k] = tot;
      tot += x;
    }
    int incl = tot;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) warpTot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      constexpr int kWarps = kPermThreads / 32;
      const int w = lane < kWarps ? warpTot[lane] : 0;
      int wi = w;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, wi, d);
        if (lane >= d) wi += y;
      }
      if (lane < kWarps) warpTot[lane] = wi - w;
    }
    __syncthreads();
    const int off = warpTot[warp] + incl - tot;
#pragma unroll
    for (int k = 0; k < kPerThread / 4; ++k)
      c4[k] = make_int4(off + v[4 * k], off + v[4 * k + 1], off + v[4 * k + 2], off + v[4 * k + 3]);
  }
  __syncthreads();
  if (ids) {
    for (int e = tid; e < L; e += kPermThreads) {
      const int pos = atomicAdd(&cnt[sId[e]], 1);
      sA[pos] = (uint16_t)e;
    }
  } else {
    for (int g = tid; g < groups; g += kPermThreads) {
      const uint4 w = philox4x32_10(make_uint4((uint32_t)g, perm, A.pair_id, tagB), k0, k1);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = 8 * g + q;
        if (e < L) {
          const int pos = atomicAdd(&cnt[bucket_in(w, e)], 1);
          sA[pos] = (uint16_t)e;
        }
      }
    }
  }
  __syncthreads();
  // cnt[b] now holds the end of bucket b.  Canonical (increasing) order
  // inside bucket b, then the forward Fisher-Yates pass from the bucket's
  // own stream.
  auto shuffle_bucket = [&](int b, int s0, int sz) {
    uint16_t* a = sA + s0;
    for (int i = 1; i < sz; ++i) {
      uint16_t key = a[i];
      int j = i - 1;
      while (j >= 0 && a[j] > key) {
        a[j + 1] = a[j];
        --j;
      }
      a[j + 1] = key;
    }
    PhiloxStream st;
    st.ctr = make_uint4(0u, perm, A.pair_id, 0x20000000u | (A.list_tag << 24) | (uint32_t)b);
    st.k0 = k0;
    st.k1 = k1;
    st.used = 4;
    for (int i = 1; i < sz; ++i) {
      const uint32_t j = st.bounded((uint32_t)(i + 1));
      const uint16_t tmp = a[i];
      a[i] = a[j];
      a[j] = tmp;
    }
  };
  if (rows) {
    // Labels only: the search sees each grid row's multiset of labels, and a
    // bucket inside one row gives the same multisets in any order (the sort
    // and the Fisher-Yates pass only decide which of its elements fall on
    // which side of a row start).  So only the buckets with a row start
    // strictly inside are shuffled: each row start finds the bucket of the
    // element the scatter put there, and the lowest row start inside a
    // bucket takes it.  (Positions past the last row form one more range.)
    // Returns (bucket, start), or bucket -1.
    auto claim = [&](int r, int u) -> int2 {
      const int p = u == 0 ? rs0 : u == 1 ? rs1 : __ldg(A.rowstart + r);
      if (p <= 0 || p >= L) return make_int2(-1, 0);
      const int lo = ids ? (int)sId[sA[p]] : bucket_of(sA[p]);
      const int s0 = lo == 0 ? 0 : cnt[lo - 1];
      if (s0 >= p) return make_int2(-1, 0);  // p starts the bucket
      const int prev = u == 0 ? rsPrev0 : u == 1 ? rsPrev1 : __ldg(A.rowstart + r - 1);
      if (r > 0 && prev > s0) return make_int2(-1, 0);  // a lower row start takes it
      return make_int2(lo, s0);
    };
    const int2 cl0 = tid <= A.n1 ? claim(tid, 0) : make_int2(-1, 0);
    const int2 cl1 = r1 <= A.n1 ? claim(r1, 1) : make_int2(-1, 0);
    if (ids && A.n1 + 1 > kPermThreads) {
      // Some threads hold two row starts: the claimed buckets go to a list
      // (in the counters, which nothing reads after the claims) so that no
      // thread shuffles two.  Entry: (start | bucket << 16, size); at most
      // 2 * kPermThreads entries of two ints, within the kBuckets counters.
      const int e0 = cl0.x >= 0 ? cnt[cl0.x] : 0, e1 = cl1.x >= 0 ? cnt[cl1.x] : 0;
      if (tid == 0) nClaim = 0;
      __syncthreads();  // every claim has read the buckets and the counters
      stage_labels();
      const unsigned m0 = __ballot_sync(0xffffffffu, cl0.x >= 0), m1 = __ballot_sync(0xffffffffu, cl1.x >= 0);
      int base = 0;
      if (lane == 0 && (m0 | m1)) base = atomicAdd(&nClaim, __popc(m0) + __popc(m1));
      base = __shfl_sync(0xffffffffu, base, 0);
      const unsigned lt = (1u << lane) - 1u;
      int2* list = reinterpret_cast<int2*>(cnt);
      if (cl0.x >= 0) list[base + __popc(m0 & lt)] = make_int2(cl0.y | (cl0.x << 16), e0 - cl0.y);
      if (cl1.x >= 0) list[base + __popc(m0) + __popc(m1 & lt)] = make_int2(cl1.y | (cl1.x << 16), e1 - cl1.y);
      __syncthreads();
      const int nc = nClaim;
      for (int k = tid; k < nc; k += kPermThreads) {
        const int2 c = list[k];
        shuffle_bucket(c.x >> 16, c.x & 0xFFFF, c.y);
      }
    } else {
      if (ids) {
        __syncthreads();  // every claim has read the buckets: the labels may come
        stage_labels();
      }
      if (cl0.x >= 0) shuffle_bucket(cl0.x, cl0.y, cnt[cl0.x] - cl0.y);
      if (cl1.x >= 0) shuffle_bucket(cl1.x, cl1.y, cnt[cl1.x] - cl1.y);
      for (int r = tid + 2 * kPermThreads, u = 2; r <= A.n1; r += kPermThreads, ++u) {
        const int2 c = claim(r, u);
        if (c.x >= 0) shuffle_bucket(c.x, c.y, cnt[c.x] - c.y);
      }
    }
  } else {
    if (ids) {
      __syncthreads();  // every scatter has read the buckets
      stage_labels();
    }
    for (int b = tid; b < kBuckets; b += kPermThreads) {
      const int s0 = b == 0 ? 0 : cnt[b - 1];
      const int sz = cnt[b] - s0;
      if (sz >= 2) shuffle_bucket(b, s0, sz);
    }
  }
  if (asyncY && A.X) asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  if (A.X) {
    int16_t* xo = A.X + (long long)blockIdx.x * A.xstride;
    if ((reinterpret_cast<uintptr_t>(xo) & 15) == 0 && (A.xstride & 7) == 0) {
      // eight labels per 16-byte store; the row's padding past L gets -1
      const int chunks = (L + 7) >> 3;
      for (int c = tid; c < chunks; c += kPermThreads) {
        const uint4 ix = reinterpret_cast<const uint4*>(sA)[c];
        const uint32_t iw[4] = {ix.x, ix.y, ix.z, ix.w};
        uint32_t ow[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int p = 8 * c + 2 * k;
          const int i0 = iw[k] & 0xFFFF, i1 = iw[k] >> 16;
          const int16_t v0 = p < L ? (sY ? sY[i0] : __ldg(A.Ylab + i0)) : (int16_t)-1;
          const int16_t v1 = p + 1 < L ? (sY ? sY[i1] : __ldg(A.Ylab + i1)) : (int16_t)-1;
          ow[k] = (uint32_t)(uint16_t)v0 | ((uint32_t)(uint16_t)v1 << 16);
        }
        reinterpret_cast<uint4*>(xo)[c] = make_uint4(ow[0], ow[1], ow[2], ow[3]);
      }
    } else if (sY) {
      for (int p = tid; p < L; p += kPermThreads) xo[p] = sY[sA[p]];
    } else {
      for (int p = tid; p < L; p += kPermThreads) xo[p] = __ldg(A.Ylab + sA[p]);
    }
  }
  if (A.sigma) {
    int* so = A.sigma + (long long)blockIdx.x * A.sstride;
    for (int p = tid; p < L; p += kPermThreads) so[p] = sA[p];
  }
}

template <int kPermThreads>
__global__ void __launch_bounds__(kPermThreads) perm_kernel(const PermArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* cnt = reinterpret_cast<int*>(smem_raw);
  uint16_t* sA = reinterpret_cast<uint16_t*>(cnt + kBuckets);
  int16_t* sY = A.stage ? reinterpret_cast<int16_t*>(smem_raw + perm_base_smem(A.L)) : nullptr;
  perm_body<kPermThreads>(A, cnt, sA, sY);
}

// X[p1] = label of the list-2 position holding the feature at list-1 position
// p1: the permuted view of list 1 puts feature idx1[p1] at p1
// (src/collections/permuted.rs:90-101); that feature sits at list-2 original
// position q = map12[idx1[p1]], which the list-2 view shows at the position
// p2 with idx2[p2] = q.
__global__ void __launch_bounds__(1024) compose_kernel(const ComposeArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint16_t* inv2 = reinterpret_cast<uint16_t*>(smem_raw);
  const int* idx1 = A.idx1 + (long long)blockIdx.x * A.stride;
  if (A.idx2) {
    const int* idx2 = A.idx2 + (long long)blockIdx.x * A.stride;
    for (int p = threadIdx.x; p < A.N2; p += blockDim.x) inv2[__ldg(idx2 + p)] = (uint16_t)p;
  }
  __syncthreads();
  int16_t* xo = A.X + (long long)blockIdx.x * A.xstride;
  for (int p = threadIdx.x; p < A.N1; p += blockDim.x) {
    int q = __ldg(A.map12 + __ldg(idx1 + p));
    int16_t lab = -1;
    if (q >= 0) lab = __ldg(A.lab2 + (A.idx2 ? (int)inv2[q] : q));
    xo[p] = lab;
  }
}

// hypergeometric_pvalue for a batch of (N, K, n, k) quadruples.
__global__ void sf_batch_kernel(const double2* __restrict__ LF, const long long* __restrict__ q,
                                double* __restrict__ out, long long count) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  out[t] = sf64(LF, q[4 * t], q[4 * t + 1], q[4 * t + 2], q[4 * t + 3]);
}

size_t grid_smem_bytes(int C, int n1, long long Npop, int smemF) {
  size_t f = smemF ? (size_t)(((Npop + 1 + 3) & ~3LL)) * 4 : 0;
  return f + (size_t)((n1 + 1 + 3) & ~3) * 4 + (size_t)kGridWarps * grid_warp_ints(C) * 4;
}

cudaError_t launch_grid(const GridArgs& a, int ctas, cudaStream_t s) {
  size_t smem = grid_smem_bytes(a.P.C, a.P.n1, a.P.Npop, a.smemF);
  switch (a.P.C) {
#define DTO_CASE(CC) \
  case CC:           \
    return launch_grid_c##CC(a, ctas, smem, s);
    DTO_FOR_EACH_C(DTO_CASE)
#undef DTO_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

size_t table_smem_bytes(int C, int n1, int n2, long long Npop, int smemF) {
  const size_t f = smemF ? (size_t)((Npop + 1 + 3) & ~3LL) * 4 : 0;
  const size_t base = f + (size_t)((n1 + 1 + 3) & ~3) * 4 + (size_t)((n2 + 3) & ~3) * 4;  // n1 = -1, n2 = 0: none
  return base + (size_t)kTableWarps * hw_warp_ints(2 * C) * 4;
}

size_t table_entries(int C, int n1) { return (size_t)n1 * 16 * hw_cq(2 * C); }

cudaError_t launch_table_build(const TableArgs& a, int nsm, cudaStream_t s) {
  long long cells = (long long)a.n1 * 16 * table_cq(a.C) / 2;  // a thread per pair of entries
  int threads = 128;
  long long blocks = std::min<long long>((cells + threads - 1) / threads, (long long)nsm * 64);
  table_build_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_table_grid(const TableGridArgs& a, int C, int ctas, cudaStream_t s) {
  // several pairs (segments): no pair tables in shared memory
  size_t smem = a.segs ? table_smem_bytes(C, -1, 0, 0, 0)
                       : table_smem_bytes(C, a.P.n1, a.P.n2, a.P.Npop, a.smemF);
  switch (C) {
#define DTO_CASE(CC) \
  case CC:           \
    return launch_table_grid_c##CC(a, ctas, smem, s);
    DTO_FOR_EACH_C(DTO_CASE)
#undef DTO_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t raise_smem_limit(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  size_t& cur = limit[std::make_pair(dev, kernel)];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

// Shared memory of a permutation launch: the counters and the indices, and
// the bucket / label area where it fits.  CTAs of 512 threads, two to an SM
// where the shared memory allows; where only one fits, CTAs of 1024 threads
// keep the SM's warps busy.
cudaError_t launch_perm(const PermArgs& a0, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  PermArgs a = a0;
  a.stage = perm_stage_area(a.L) ? 1 : 0;
  const size_t smem = perm_base_smem(a.L) + (a.stage ? perm_round16((size_t)a.L * 2) : 0);
  cudaError_t e = raise_smem_limit((const void*)perm_kernel<512>, smem);
  int n = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, perm_kernel<512>, 512, smem);
  if (e != cudaSuccess) return e;
  if (n >= 2) {
    perm_kernel<512><<<count, 512, smem, s>>>(a);
  } else {
    e = raise_smem_limit((const void*)perm_kernel<1024>, smem);
    if (e != cudaSuccess) return e;
    perm_kernel<1024><<<count, 1024, smem, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_compose(const ComposeArgs& a, int count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  size_t smem = a.idx2 ? (((size_t)a.N2 * 2 + 15) & ~(size_t)15) : 16;
  cudaError_t e = raise_smem_limit((const void*)compose_kernel, smem);
  if (e != cudaSuccess) return e;
  compose_kernel<<<count, 1024, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sf_batch(const double2* LF, const long long* q, double* out, long long count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  int threads = 128;
  long long blocks = (count + threads - 1) / threads;
  sf_batch_kernel<<<(unsigned)blocks, threads, 0, s>>>(LF, q, out, count);
  return cudaGetLastError();
}

}  // namespace dto
