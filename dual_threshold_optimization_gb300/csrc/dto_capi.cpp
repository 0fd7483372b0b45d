// dto_capi.cpp -- host side of libdto.so: contexts, list pairs and the C ABI
// declared in include/dto.h (the permutation-null driver is dto_lane.cpp,
// the request executor dto_serve.cpp).
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

#include "dto_host.h"

using namespace dto;

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

// round(x * scale) of a double-double x, to the nearest integer; scale is a
// power of two (2^f), so the products are exact (as ldexp's are, at a sixth
// of the cost: the table has population + 1 entries per pair).
long long dd_round_scaled(double hi, double lo, double scale) {
  double x = hi * scale, y = lo * scale;
  double r = std::nearbyint(x);
  double frac = (x - r) + y;
  if (frac > 0.5) r += 1.0;
  else if (frac < -0.5) r -= 1.0;
  return (long long)r;
}

int ensure_lf(dto_ctx* ctx, long long nmax) {
  std::lock_guard<std::mutex> g(ctx->lf_mu);
  if (nmax <= ctx->lf_cap) return DTO_OK;
  long long cap = std::max(nmax, 2 * ctx->lf_cap);
  cap = std::max(cap, 1024LL);
  lf_table_dd(cap, ctx->lf_hi, ctx->lf_lo);
  std::vector<double2> h((size_t)cap + 1);
  for (size_t m = 0; m <= (size_t)cap; ++m) h[m] = make_double2(ctx->lf_hi[m], ctx->lf_lo[m]);
  double2* d = nullptr;
  CK(cudaMalloc(&d, h.size() * sizeof(double2)));
  cudaError_t e = cudaMemcpy(d, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_err(ctx, e, "log-factorial table upload");
  }
  // kernels of other lanes may still read the old table: retire it, do not free it
  double2* old = ctx->dLF.exchange(d);
  if (old) ctx->lf_old.push_back(old);
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

// The pair argument of an entry point: present and created on this context.
int pair_check(dto_ctx* ctx, const dto_pair* P, const char* fn) {
  if (!ctx) return DTO_ERR_INVALID;
  if (!P) return set_err(ctx, DTO_ERR_INVALID, std::string(fn) + ": null pair");
  if (P->ctx != ctx) return set_err(ctx, DTO_ERR_INVALID, std::string(fn) + ": the pair belongs to another context");
  return DTO_OK;
}

int pick_C(int n2) {
  for (int c : kCs)
    if (32 * c >= n2) return c;
  return -1;
}

}  // namespace

namespace {

// Stable sort by rank (src/collections/ranked.rs:527-542): a counting sort
// when the ranks are dense, else a byte-wise LSD radix sort; both keep equal
// ranks in input order, as the reference's stable comparison sort does.
void rank_order(const uint32_t* r, int64_t n, std::vector<int32_t>& order) {
  order.resize((size_t)n);
  if (n == 0) return;
  uint32_t mx = 0;
  for (int64_t q = 0; q < n; ++q) mx = std::max(mx, r[q]);
  if ((uint64_t)mx <= 4 * (uint64_t)n + 1024) {
    std::vector<int64_t> at((size_t)mx + 2, 0);  // at[v]: first slot of rank v
    for (int64_t q = 0; q < n; ++q) ++at[(size_t)r[q] + 1];
    for (size_t v = 1; v < at.size(); ++v) at[v] += at[v - 1];
    for (int64_t q = 0; q < n; ++q) order[(size_t)at[r[q]]++] = (int32_t)q;
    return;
  }
  std::vector<int32_t> tmp((size_t)n);
  for (int64_t q = 0; q < n; ++q) order[(size_t)q] = (int32_t)q;
  for (int shift = 0; shift < 32 && (mx >> shift) != 0; shift += 8) {
    int64_t at[257] = {0};
    for (int64_t q = 0; q < n; ++q) ++at[((r[order[(size_t)q]] >> shift) & 255u) + 1];
    for (int d = 1; d <= 256; ++d) at[d] += at[d - 1];
    for (int64_t q = 0; q < n; ++q) {
      const int32_t e = order[(size_t)q];
      tmp[(size_t)at[(r[e] >> shift) & 255u]++] = e;
    }
    order.swap(tmp);
  }
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
    case DTO_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

int dto_ctx_create(int device, dto_ctx** out) {
  if (!out) return DTO_ERR_INVALID;
  *out = nullptr;
  dto_ctx* ctx = new dto_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  cudaDeviceProp prop;
  if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete ctx;
    return e == cudaErrorMemoryAllocation ? DTO_ERR_OOM : DTO_ERR_CUDA;
  }
  ctx->nsm = prop.multiProcessorCount;
  // dynamic shared memory a kernel may take: the per-block limit less 1 KB
  // for the kernels' static shared arrays
  ctx->smem_optin = prop.sharedMemPerBlockOptin - 1024;
  const int rc = lane_create(ctx, &ctx->lane0, &ctx->err);
  if (rc) {
    delete ctx;
    return rc;
  }
  // a new pair of the shape of an earlier one starts from that pair's ladder
  // (LadderModel): its first run skips the exhaustive first batch
  ctx->lane0->use_model = true;
  *out = ctx;
  return DTO_OK;
}

int dto_ctx_destroy(dto_ctx* ctx) {
  if (!ctx) return DTO_ERR_INVALID;
  cudaSetDevice(ctx->device);
  lane_destroy(ctx->lane0);
  cudaFree(ctx->dLF.load());
  for (double2* d : ctx->lf_old) cudaFree(d);
  delete ctx;
  return DTO_OK;
}

const char* dto_last_error(const dto_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* dto_ctx_stream(dto_ctx* ctx) { return ctx ? (void*)ctx->lane0->stream : nullptr; }

int dto_rank_order(const uint32_t* ranks, int64_t n, int32_t* order) {
  if (n < 0 || n > 0x7fffffffLL || (n > 0 && (!ranks || !order))) return DTO_ERR_INVALID;
  std::vector<int32_t> o;
  rank_order(ranks, n, o);
  std::copy(o.begin(), o.end(), order);
  return DTO_OK;
}

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
  P->serial = ctx->next_serial.fetch_add(1);
  P->pair_id = 0;  // Philox stream id; dto_pair_set_stream changes it
  P->N1 = n1;
  P->N2 = n2;
  P->npop = population;
  P->nfeat = n_features;
  rank_order(ranks1, n1, P->order1);
  rank_order(ranks2, n2, P->order2);
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
  // m_j: list-1 positions whose feature sits in list 2 at a rank <= T2[j]
  std::vector<int> mcnt((size_t)nt2, 0);
  for (int64_t p = 0; p < n1; ++p) {
    int q = pos2[(size_t)P->f1[(size_t)p]];
    P->map12[(size_t)p] = q;
    if (q >= 0) {
      ++common;
      P->ylab[(size_t)p] = P->lab2[(size_t)q];
      const int16_t l = P->lab2[(size_t)q];
      if (l >= 0) ++mcnt[(size_t)((l / Cp) * P->C + (l % Cp))];
    }
  }
  for (int j = 1; j < nt2; ++j) mcnt[(size_t)j] += mcnt[(size_t)j - 1];
  // the same labels in the table sweep's form (the labels a table run
  // draws), through a table over the grid kernel's labels
  std::vector<int16_t> g2h((size_t)32 * Cp, -1);
  for (int j = 0; j < 32 * P->C; ++j) g2h[(size_t)grid_label_of_column(j, P->C)] = (int16_t)hw_label_of_column(j, P->C);
  auto to_hw = [&](const std::vector<int16_t>& g) {
    std::vector<int16_t> v(g.size(), -1);
    for (size_t q = 0; q < g.size(); ++q)
      if (g[q] >= 0) v[q] = g2h[(size_t)g[q]];
    return v;
  };
  const std::vector<int16_t> ylabHw = to_hw(P->ylab), lab2Hw = to_hw(P->lab2);
  P->ncommon = common;
  P->same_set = (common == n1 && common == n2);
  // fixed-point fraction bits: |ln pmf| <= N ln 2 must fit in int32 with slack
  int f = 0;
  while (f < 24 && ((double)population * 0.6931471805599453 + 64.0) * std::ldexp(1.0, f + 1) < 2.0e9) ++f;
  P->fshift = f;
  int rc = ensure_lf(ctx, population);
  if (rc) { delete P; return rc; }
  std::vector<uint32_t> F((size_t)population + 1);
  const double fscale = std::ldexp(1.0, f);
  for (long long m = 0; m <= population; ++m)
    F[(size_t)m] = (uint32_t)(unsigned long long)dd_round_scaled(ctx->lf_hi[(size_t)m], ctx->lf_lo[(size_t)m], fscale);
  std::vector<int> row((size_t)nt1 + 1);
  row[0] = 0;
  for (int i = 0; i < nt1; ++i) row[(size_t)i + 1] = P->c1[(size_t)i];
  // the pair's device arrays: one allocation and one copy, each array on a
  // 256-byte boundary
  struct Part {
    const void* h;
    size_t bytes;
    void** d;
  };
  const Part parts[9] = {{row.data(), row.size() * 4, (void**)&P->dRow},
                         {P->c2.data(), P->c2.size() * 4, (void**)&P->dNcnt},
                         {F.data(), F.size() * 4, (void**)&P->dF},
                         {P->ylab.data(), P->ylab.size() * 2, (void**)&P->dYlab},
                         {P->lab2.data(), P->lab2.size() * 2, (void**)&P->dLab2},
                         {P->map12.data(), P->map12.size() * 4, (void**)&P->dMap12},
                         {mcnt.data(), mcnt.size() * 4, (void**)&P->dMcnt},
                         {ylabHw.data(), ylabHw.size() * 2, (void**)&P->dYlabHw},
                         {lab2Hw.data(), lab2Hw.size() * 2, (void**)&P->dLab2Hw}};
  constexpr int kParts = (int)(sizeof(parts) / sizeof(parts[0]));
  size_t off[kParts], total = 0;
  for (int k = 0; k < kParts; ++k) {
    off[k] = total;
    total += (parts[k].bytes + 255) & ~(size_t)255;
    P->upload_bytes += (long long)parts[k].bytes;
  }
  std::vector<unsigned char> host(total, 0);
  for (int k = 0; k < kParts; ++k)
    if (parts[k].bytes) std::memcpy(host.data() + off[k], parts[k].h, parts[k].bytes);
  cudaError_t e = cudaMalloc(&P->dBase, std::max(total, (size_t)256));
  if (e == cudaSuccess) {
    for (int k = 0; k < kParts; ++k) *parts[k].d = static_cast<unsigned char*>(P->dBase) + off[k];
    e = cudaMemcpyAsync(P->dBase, host.data(), total, cudaMemcpyHostToDevice, ctx->lane0->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->lane0->stream);
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
  cudaFree(P->dBase);
  for (uint16_t* t : P->dWaveKthr) cudaFree(t);
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

int dto_pair_set_ladder(dto_pair* P, const double* minp, int64_t count) {
  if (!P || count < 0 || (count > 0 && !minp)) return DTO_ERR_INVALID;
  std::vector<double> v;
  v.reserve((size_t)count);
  for (int64_t q = 0; q < count; ++q) {
    if (!(minp[q] >= 0.0 && minp[q] <= 1.0)) return set_err(P->ctx, DTO_ERR_INVALID, "dto_pair_set_ladder: p-values must lie in [0, 1]");
    v.push_back(minp[q]);
  }
  std::lock_guard<std::mutex> g(P->ladder_mu);
  P->ladder_pending = false;  // a ladder left by the last run gives way
  if (count == 0) {
    P->ladder_ok = false;
    P->ladder_sample.clear();
    return DTO_OK;
  }
  ladder_of(v, P->fshift, P->ladder_tau, P->q0);
  P->ladder_ok = true;
  P->ladder_sample = v;
  return DTO_OK;
}

int dto_pair_set_level0_quantile(dto_pair* P, double q0) {
  if (!P) return DTO_ERR_INVALID;
  if (!(q0 >= 0.5 && q0 <= 0.99))
    return set_err(P->ctx, DTO_ERR_INVALID, "dto_pair_set_level0_quantile: the quantile must lie in [0.5, 0.99]");
  ladder_flush(P->ctx, P);
  std::lock_guard<std::mutex> g(P->ladder_mu);
  P->q0 = q0;
  // the ladder again from the last run's sample, at the new quantile
  if (P->ladder_ok && !P->ladder_sample.empty()) ladder_of(P->ladder_sample, P->fshift, P->ladder_tau, q0);
  return DTO_OK;
}

int dto_pair_tune(dto_ctx* ctx, dto_pair* P, int64_t n_perm, uint64_t seed, double* best_quantile) {
  if (int rc = pair_check(ctx, P, "dto_pair_tune")) return rc;
  if (n_perm <= 1024 || n_perm > 0x7fffffffLL)
    return set_err(ctx, DTO_ERR_INVALID,
                   "dto_pair_tune: n_perm must take the table ladder (more than 1,024 permutations)");
  // the candidates' timed runs, on the context's own lane: one run first
  // (the ladder, the kernels loaded), then three runs per candidate, all of
  // the same permutations (run-to-run differences of the permutations are as
  // large as the candidates' differences), the first rebuilding the tables
  // and the fastest device time of the other two counted
  static const double kCandidates[3] = {0.80, 0.85, 0.90};
  std::vector<double> minp((size_t)n_perm);
  dto_result unperm{};
  dto_summary sum{};
  auto run = [&](uint64_t s) -> int {
    std::lock_guard<std::mutex> g(ctx->mu);
    return lane_run_range(ctx->lane0, P, 1u, n_perm, s, nullptr, DTO_PRECISION_SCREEN, &unperm, minp.data(),
                          nullptr, &sum);
  };
  int rc = run(seed);
  if (rc) return rc;
  double best_q = 0.0, best_ms = 1e300;
  for (double q : kCandidates) {
    rc = dto_pair_set_level0_quantile(P, q);
    if (rc) return rc;
    double ms = 1e300;
    for (int r = 0; r < 3; ++r) {
      rc = run(seed + 1);
      if (rc) return rc;
      if (r > 0) ms = std::min(ms, sum.device_ms);
    }
    if (ms < best_ms) {
      best_ms = ms;
      best_q = q;
    }
  }
  rc = dto_pair_set_level0_quantile(P, best_q);
  if (rc) return rc;
  {
    // pairs of this shape start with it (LadderModel)
    std::lock_guard<std::mutex> g(P->ladder_mu);
    LadderShape x = shape_of(P);
    for (int l = 0; l < kLadderTaus; ++l) x.nats[l] = std::ldexp((double)P->ladder_tau[l], -P->fshift);
    x.q0 = best_q;
    ctx->ladders.record(x);
  }
  if (best_quantile) *best_quantile = best_q;
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
  if (int rc = pair_check(ctx, P, "dto_run_range")) return rc;
  std::lock_guard<std::mutex> g(ctx->mu);
  return lane_run_range(ctx->lane0, P, perm_first, n_perm, seed, perm_idx, precision, out_unpermuted, out_minp,
                        out_perm, out_summary);
}

int dto_optimize(dto_ctx* ctx, dto_pair* P, int permute, uint64_t seed, uint32_t perm_id, const int32_t* idx1,
                 const int32_t* idx2, int precision, dto_result* out) {
  if (int rc = pair_check(ctx, P, "dto_optimize")) return rc;
  if (!out) return set_err(ctx, DTO_ERR_INVALID, "dto_optimize: null out");
  if (precision != DTO_PRECISION_FP64 && precision != DTO_PRECISION_SCREEN)
    return set_err(ctx, DTO_ERR_INVALID, "unknown precision");
  std::lock_guard<std::mutex> g(ctx->mu);
  Lane* L = ctx->lane0;
  CK(cudaSetDevice(ctx->device));
  const int mode = precision == DTO_PRECISION_FP64 ? kModeFull64 : kModeScreen;
  int rc = lane_grow(L, &L->dRes, &L->resBytes, 2 * sizeof(TaskResult));
  if (rc) return rc;
  rc = lane_grow_host(L, &L->hRes, &L->hResBytes, 2 * sizeof(TaskResult));
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
      CK(cudaMemcpyAsync(dIdx, idx1, (size_t)P->N1 * 4, cudaMemcpyHostToDevice, L->stream));
      CK(cudaMemcpyAsync((int32_t*)dIdx + P->N1, idx2, (size_t)P->N2 * 4, cudaMemcpyHostToDevice, L->stream));
      dI = (const int32_t*)dIdx;
    }
    rc = lane_make_labels(L, P, seed, perm_id, 1, dI);
    if (rc) return rc;
    dX = (const int16_t*)L->dX;
  }
  rc = lane_grid_tasks(L, P, dX, xstride_of(P->N1), 1, mode, (TaskResult*)L->dRes);
  if (rc) return rc;
  CK(cudaMemcpyAsync(L->hRes, L->dRes, sizeof(TaskResult), cudaMemcpyDeviceToHost, L->stream));
  CK(cudaStreamSynchronize(L->stream));
  const TaskResult r = ((TaskResult*)L->hRes)[0];
  if (r.i < 0 || r.i >= (int)P->T1.size() || r.j < 0 || r.j >= (int)P->T2.size())
    return set_err(ctx, DTO_ERR_CUDA, "dto_optimize: the search returned no grid cell");
  fill_result(P, r, permute ? 1 : 0, out);
  return DTO_OK;
}

int dto_grid_dump(dto_ctx* ctx, dto_pair* P, const int32_t* idx1, const int32_t* idx2, dto_result* records) {
  if (int rc = pair_check(ctx, P, "dto_grid_dump")) return rc;
  if (!records) return set_err(ctx, DTO_ERR_INVALID, "dto_grid_dump: null records");
  std::lock_guard<std::mutex> g(ctx->mu);
  Lane* L = ctx->lane0;
  CK(cudaSetDevice(ctx->device));
  const long long ncell = (long long)P->T1.size() * (long long)P->T2.size();
  int rc = lane_grow(L, &L->dRes, &L->resBytes, 2 * sizeof(TaskResult));
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
    CK(cudaMemcpyAsync(dIdx, idx1, (size_t)P->N1 * 4, cudaMemcpyHostToDevice, L->stream));
    CK(cudaMemcpyAsync((int32_t*)dIdx + P->N1, idx2, (size_t)P->N2 * 4, cudaMemcpyHostToDevice, L->stream));
    rc = lane_make_labels(L, P, 0, 0, 1, (const int32_t*)dIdx);
    if (rc) return rc;
    dX = (const int16_t*)L->dX;
  }
  rc = lane_grid_tasks(L, P, dX, xstride_of(P->N1), 1, kModeDump, (TaskResult*)L->dRes, (int*)dK, (double*)dP);
  if (rc) return rc;
  std::vector<int> hk((size_t)ncell);
  std::vector<double> hp((size_t)ncell);
  CK(cudaMemcpyAsync(hk.data(), dK, (size_t)ncell * 4, cudaMemcpyDeviceToHost, L->stream));
  CK(cudaMemcpyAsync(hp.data(), dP, (size_t)ncell * 8, cudaMemcpyDeviceToHost, L->stream));
  CK(cudaStreamSynchronize(L->stream));
  const int permuted = (idx1 && idx2) ? 1 : 0;
  const long long nt2 = (long long)P->T2.size();
  for (long long c = 0; c < ncell; ++c) {
    TaskResult r{hp[(size_t)c], (int)(c / nt2), (int)(c % nt2), hk[(size_t)c], DTO_ROUTE_FP64};
    fill_result(P, r, permuted, &records[c]);
  }
  return DTO_OK;
}

int dto_hypergeom_sf(dto_ctx* ctx, const int64_t* N, const int64_t* K, const int64_t* n, const int64_t* k,
                     double* out, int64_t count) {
  if (!ctx || count < 0 || (count > 0 && (!N || !K || !n || !k || !out))) return set_err(ctx, DTO_ERR_INVALID, "null argument");
  if (count == 0) return DTO_OK;
  std::lock_guard<std::mutex> g(ctx->mu);
  Lane* L = ctx->lane0;
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
  CK(cudaMemcpyAsync(dq, q.data(), q.size() * 8, cudaMemcpyHostToDevice, L->stream));
  CK(launch_sf_batch(ctx->dLF.load(), (const long long*)dq, (double*)dout, count, L->stream));
  CK(cudaMemcpyAsync(out, dout, (size_t)count * 8, cudaMemcpyDeviceToHost, L->stream));
  CK(cudaStreamSynchronize(L->stream));
  return DTO_OK;
}

int dto_export_permutations(dto_ctx* ctx, dto_pair* P, uint64_t seed, uint32_t perm_first, int64_t count,
                            int32_t* idx1, int32_t* idx2) {
  if (int rc = pair_check(ctx, P, "dto_export_permutations")) return rc;
  if (count < 0 || (count > 0 && (!idx1 || !idx2)))
    return set_err(ctx, DTO_ERR_INVALID, "dto_export_permutations: null argument");
  if (count == 0) return DTO_OK;
  std::lock_guard<std::mutex> g(ctx->mu);
  Lane* L = ctx->lane0;
  CK(cudaSetDevice(ctx->device));
  int rc = lane_grow(L, &L->dSig, &L->sigBytes, (size_t)count * (P->N1 + P->N2) * 4);
  if (rc) return rc;
  int* sig = (int*)L->dSig;
  PermArgs a{};
  a.seed = seed;
  a.pair_id = P->pair_id;
  a.perm_base = perm_first;
  a.L = (int)P->N1;
  a.list_tag = 1;
  a.sigma = sig;
  a.sstride = P->N1;
  CK(launch_perm(a, (int)count, L->stream));
  if (!P->same_set) {
    a.L = (int)P->N2;
    a.list_tag = 2;
    a.sigma = sig + count * P->N1;
    a.sstride = P->N2;
    CK(launch_perm(a, (int)count, L->stream));
  }
  CK(cudaMemcpyAsync(idx1, sig, (size_t)count * P->N1 * 4, cudaMemcpyDeviceToHost, L->stream));
  if (!P->same_set)
    CK(cudaMemcpyAsync(idx2, sig + count * P->N1, (size_t)count * P->N2 * 4, cudaMemcpyDeviceToHost, L->stream));
  CK(cudaStreamSynchronize(L->stream));
  if (P->same_set)
    for (int64_t b = 0; b < count; ++b)
      for (int64_t p = 0; p < P->N2; ++p) idx2[b * P->N2 + p] = (int32_t)p;
  return DTO_OK;
}

int dto_run_range_noalloc(dto_ctx* ctx, dto_pair* P, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                          double* d_minp) {
  if (int rc = pair_check(ctx, P, "dto_run_range_noalloc")) return rc;
  if (n_perm < 0 || (n_perm > 0 && !d_minp))
    return set_err(ctx, DTO_ERR_INVALID, "dto_run_range_noalloc: null argument");
  if ((long long)perm_first + n_perm > 0xffffffffLL)
    return set_err(ctx, DTO_ERR_INVALID, "dto_run_range_noalloc: permutation ids out of range");
  std::lock_guard<std::mutex> g(ctx->mu);
  Lane* L = ctx->lane0;
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
    // only each grid row's multiset of labels reaches the search, so buckets
    // that lie inside one row keep their order, as in a dto_run_range run
    a.rowstart = P->dRow;
    a.n1 = P->dev.n1;
    CK(launch_perm(a, cnt, L->stream));
  } else {
    const long long ss = P->N1 + P->N2;
    a.L = (int)P->N1;
    a.list_tag = 1;
    a.sigma = sig;
    a.sstride = ss;
    CK(launch_perm(a, cnt, L->stream));
    a.L = (int)P->N2;
    a.list_tag = 2;
    a.sigma = sig + P->N1;
    CK(launch_perm(a, cnt, L->stream));
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
    CK(launch_compose(c, cnt, L->stream));
  }
  CK(cudaMemsetAsync(work, 0, 256, L->stream));  // the shared task counter starts at zero
  GridArgs gk{};
  gk.P = P->dev;
  gk.P.LF = ctx->dLF.load();
  gk.X = X;
  gk.xstride = xs;
  gk.ntask = cnt;
  gk.mode = kModeScreen;
  gk.route = DTO_ROUTE_SCREEN;
  gk.smemF = grid_smem_bytes(P->C, P->dev.n1, P->npop, 1) <= ctx->smem_optin ? 1 : 0;
  gk.out = res;
  gk.work = work;
  const int ctas = std::max(1, std::min(ctx->nsm, (cnt + kGridWarps - 1) / kGridWarps));
  CK(launch_grid(gk, ctas, L->stream));
  CK(launch_noalloc_copy_p(res, d_minp, cnt, L->stream));
  return DTO_OK;
}

}  // extern "C"
