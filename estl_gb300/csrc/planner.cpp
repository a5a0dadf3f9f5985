// planner.cpp — see planner.h.
#include "planner.h"

#include <algorithm>
#include <cstdio>

#include "bluestein_core.cuh"
#include "fft_core.cuh"
#include "bulk_core.cuh"
#include "resident_core.cuh"
#include "cluster_core.cuh"

namespace estl {

namespace {

template <class K>
TileCfg cfg_of(int kind, int logm, int loge, int logr, int logc, int pipe = 0, int tc = 0) {
  return TileCfg{kind, logm, loge, logr, logc, K::NT, (int)(K::SMEM_ELEMS * (int)sizeof(cf32)), pipe, tc,
                 cluster_of<K>::log_cluster, cluster_of<K>::log_split};
}

std::vector<TileCfg> build_configs() {
  std::vector<TileCfg> v;
#define ESTL_X_SINGLE(M, E, R, C) v.push_back(cfg_of<SingleKernel<M, E, R, C>>(STEP_SINGLE, M, E, R, C));
#define ESTL_X_COL(M, E, R, C) v.push_back(cfg_of<ColKernel<M, E, R, C>>(STEP_COL, M, E, R, C));
#define ESTL_X_ROW(M, E, R, C) v.push_back(cfg_of<RowKernel<M, E, R, C>>(STEP_ROW, M, E, R, C));
#define ESTL_X_BULK_ROW(M, E, R, C) v.push_back(cfg_of<BulkRowKernel<M, E, R, C>>(STEP_ROW, M, E, R, C, 2));
#define ESTL_X_BULK_COL(M, E, R, C) v.push_back(cfg_of<BulkColKernel<M, E, R, C>>(STEP_COL, M, E, R, C, 2));
#define ESTL_X_RES(M, E, R, H) v.push_back(cfg_of<ResKernel<M, E, R, H>>(STEP_SINGLE, M, E, R, 0, 2 + H));
#define ESTL_X_CLUSTER(N, LR, N2, E) v.push_back(cfg_of<ClusterKernel<N, LR, N2, E>>(STEP_SINGLE, N, E, 4, 0));
#define ESTL_X_COLUMN(M, E, C) v.push_back(cfg_of<ColKernel<M, E, 4, C, false, false>>(STEP_COLUMN, M, E, 4, C));
#define ESTL_X_TC_SINGLE(M, C) v.push_back(cfg_of<SingleKernel<M, 4, 4, C, true>>(STEP_SINGLE, M, 4, 4, C, 0, 1));
#define ESTL_X_TC_COL(M, C) v.push_back(cfg_of<ColKernel<M, 4, 4, C, true>>(STEP_COL, M, 4, 4, C, 0, 1));
#define ESTL_X_TC_ROW(M, C) v.push_back(cfg_of<RowKernel<M, 4, 4, C, true>>(STEP_ROW, M, 4, 4, C, 0, 1));
#include "kernel_list.inc"
  return v;
}

// Planner defaults: the configuration used before any autotuning, from
// autotuner runs on a GB300 (the tuning cache overrides them per size).
// Single kernel: 16 elements per thread and about 256 threads per CTA up to
// 2^12; 32 elements per thread (256 / 512 threads, one transform per CTA)
// for 2^13 and 2^14.
// Four-step (lengths without a tuned entry): N2 = 2^floor(log2 N / 2) column
// DFTs; column tiles as wide as 512 threads allow; row tiles of 8 rows
// (N1 <= 2^9) or 4 rows (larger); chunks of 2^27 elements (1 GiB scratch).
const TileCfg* default_single(int logm) {
  // autotuner winners on a GB300 (1 GiB batches): log2 M -> (log2 E, log2 C,
  // log2 radix); 2^13 and 2^14 run radix-32 passes (three instead of four)
  static const int tuned[][4] = {{10, 4, 1, 4}, {11, 4, 0, 4}, {12, 5, 0, 4}, {13, 5, 0, 5}, {14, 5, 0, 5}};
  for (const auto& t : tuned)
    if (t[0] == logm)
      if (const TileCfg* c = find_tile(STEP_SINGLE, logm, t[1], t[3], t[2])) return c;
  const TileCfg* best = nullptr;
  const int want_e = logm >= 13 ? 5 : std::min(4, logm);
  for (const TileCfg& c : tile_configs()) {
    if (c.kind != STEP_SINGLE || c.logm != logm || c.pipe || c.tc || c.cluster) continue;
    if (c.loge != want_e) continue;
    if (!best || std::abs(c.nthreads - 256) < std::abs(best->nthreads - 256)) best = &c;
  }
  return best;
}

// The widest E=16 tile of at most 512 threads whose chunk is at most
// 2^want_logc transforms; failing that, the narrowest chunk up to 2^max_logc.
const TileCfg* default_pass(int kind, int logm, int want_logc, int max_logc) {
  const TileCfg* best = nullptr;
  for (const TileCfg& c : tile_configs()) {
    if (c.kind != kind || c.logm != logm || c.loge != 4 || c.logc > want_logc || c.pipe || c.tc) continue;
    if (c.nthreads > 512) continue;
    if (!best || c.logc > best->logc) best = &c;
  }
  if (!best)
    for (const TileCfg& c : tile_configs()) {
      if (c.kind != kind || c.logm != logm || c.logc > max_logc || c.pipe || c.tc) continue;
      if (!best || c.logc < best->logc || (c.logc == best->logc && c.nthreads < best->nthreads)) best = &c;
    }
  return best;
}

}  // namespace

const std::vector<TileCfg>& tile_configs() {
  static const std::vector<TileCfg> v = build_configs();
  return v;
}

const TileCfg* find_tile(int kind, int logm, int loge, int logr, int logc, int pipe, int tc, int cluster,
                         int csplit) {
  for (const TileCfg& c : tile_configs())
    if (c.kind == kind && c.logm == logm && c.loge == loge && c.logr == logr && c.logc == logc && c.pipe == pipe &&
        c.tc == tc && c.cluster == cluster && c.csplit == csplit)
      return &c;
  return nullptr;
}

// Cluster tiles that single-kernel plans use by default (measured on a
// GB300, 1 GiB batches): log2 N -> (log2 CTAs per cluster, log2 N2, log2 E).
static const TileCfg* default_cluster(int logn) {
  // 2^14: 4097 vs 3955 GB/s for the single-CTA radix-32 tile; 2^15: 3566 vs
  // 3017 GB/s for the two-pass four-step; 2^16 and 2^17 stay four-step
  static const int tuned[][4] = {{14, 2, 7, 4}, {15, 3, 8, 4}};
  for (const auto& t : tuned)
    if (t[0] == logn)
      if (const TileCfg* c = find_tile(STEP_SINGLE, logn, t[3], 4, 0, 0, 0, t[1], t[2])) return c;
  return nullptr;
}

// The tensor-core tile of a kind and length (kernel_list.inc instantiates one
// per length), or the one with the requested rows / columns per CTA.
static const TileCfg* find_tc(int kind, int logm, int logc) {
  for (const TileCfg& c : tile_configs())
    if (c.tc && c.kind == kind && c.logm == logm && (logc < 0 || c.logc == logc)) return &c;
  return nullptr;
}

// Radix of a tile choice: -1 = radix 16.
static int lr_of(int logr) { return logr < 0 ? 4 : logr; }

// Which variant of a tile a step runs: ch.pipe (2 bulk-load, 3 / 4 resident)
// where that variant exists, else the plain tile.
static int use_pipe(const PlanChoice& ch, const TileCfg* c) {
  if (ch.pipe < 2) return 0;
  return find_tile(c->kind, c->logm, c->loge, c->logr, c->logc, ch.pipe) ? ch.pipe : 0;
}

int ilog2_exact(long long n) {
  if (n < 1) return -1;
  int l = 0;
  while ((1LL << l) < n) l++;
  return ((1LL << l) == n) ? l : -1;
}

static void set_err(std::string* err, const char* msg, long long a = 0, long long b = 0) {
  if (!err) return;
  char buf[256];
  std::snprintf(buf, sizeof buf, msg, a, b);
  *err = buf;
}

bool make_plan(long long n, long long batch, const PlanChoice& choice, Plan1D* out, std::string* err) {
  int logn = ilog2_exact(n);
  if (logn < 0) {
    set_err(err, "transform length %lld is not a power of two", n);
    return false;
  }
  if (logn > kMaxLogN) {
    set_err(err, "transform length 2^%lld exceeds the supported maximum 2^%lld", logn, kMaxLogN);
    return false;
  }
  if (batch < 1) {
    set_err(err, "batch must be >= 1 (got %lld)", batch);
    return false;
  }
  if (batch > ((1LL << kMaxTotalLog) >> logn)) {
    set_err(err, "n * batch must be at most 2^40 elements (got n = %lld, batch = %lld)", n, batch);
    return false;
  }
  Plan1D p;
  p.n = n;
  p.batch = batch;
  p.logn = logn;
  p.choice = choice;
  const long long total = n * batch;

  if (logn == 0) {
    Step s{STEP_COPY, 0, 0, 0, 0, 1, BUF_IN, BUF_OUT, 0, total, 0, total, total, 0};
    p.steps.push_back(s);
    p.hbm_passes = 1;
    *out = p;
    return true;
  }

  // split precision: the radix-16 passes on the tensor cores.  n < 16 has no
  // radix-16 pass and runs the FP32 tiles.
  const bool tc = choice.split != 0 && logn >= 4;
  if (choice.split < 0 || choice.split > 3) {
    set_err(err, "unknown split precision %lld", choice.split);
    return false;
  }
  if (choice.mode == 3 || choice.mode < 0 || choice.mode > 4) {
    set_err(err, "unknown plan mode %lld", choice.mode);
    return false;
  }
  if (tc && choice.pipe > 0) {
    set_err(err, "split precision runs the plain single / four-step tiles (mode %lld)", choice.mode);
    return false;
  }
  int mode = choice.mode;
  // N >= 2^23 (FP32): three passes of wide runs beat two passes whose 2^11 /
  // 2^12-point tiles leave only 2-4 columns per CTA (measured on a GB300:
  // 2023 vs 1790 GB/s at 2^23, 1987 vs 1563 GB/s at 2^24, 1 GiB batches)
  bool three_default = false;
  if (mode == 0 && !tc && logn >= kThreePassDefaultLog) {
    mode = 4;
    three_default = true;
  }
  const bool cluster_default = mode == 0 && !tc && choice.single_cluster < 0 && choice.single_loge < 0 &&
                               default_cluster(logn) != nullptr;
  if (mode == 0) mode = (logn <= (tc ? kTcSingleMaxLog : kSingleMaxLog) || cluster_default) ? 1 : 2;

  if (mode == 4) {
    // three passes, N = R * Q * P (x[n1 + P n2 + PQ n3]):
    //   A  column DFTs of length R over the PQ columns, four-step twiddle
    //      w_N^{n' k3} (n' = n1 + P n2)             in      -> out (temporary)
    //   B  per (b, k3): column DFTs of length Q over the P columns, twiddle
    //      w_{PQ}^{n1 k2}, stored as rows k3 + R k2   out     -> scratch
    //   C  row DFTs of length P, X[k3 + R k2 + RQ k1]  scratch -> out
    // Every pass moves C-wide runs of 2^7..2^9-point tiles.
    if (tc) {
      set_err(err, "split precision runs the single / four-step tiles (mode %lld)", choice.mode);
      return false;
    }
    // default split (measured): R = 2^7, Q = 2^8 from 2^23 on, P the rest
    const int lr = choice.logn2 > 0 ? choice.logn2 : 7;
    const int lq = choice.logn3 > 0 ? choice.logn3 : (logn >= 23 ? 8 : 7);
    const int lp = logn - lr - lq;
    if (lr < 7 || lr > 9 || lq < 7 || lq > 9 || lp < 7 || lp > 9) {
      set_err(err, "three-pass plan needs three DFT lengths of 2^7..2^9 (log2 N = %lld)", logn);
      return false;
    }
    static const int col_c[10] = {0, 0, 0, 0, 0, 0, 0, 5, 4, 3}, row_c[10] = {0, 0, 0, 0, 0, 0, 0, 4, 3, 2};
    auto col_for = [&](int m) -> const TileCfg* {
      if (choice.col_loge >= 0)
        if (const TileCfg* c = find_tile(STEP_COL, m, choice.col_loge, lr_of(choice.col_logr), choice.col_logc)) return c;
      return find_tile(STEP_COL, m, 4, 4, col_c[m]);
    };
    const TileCfg* ca = col_for(lr);
    const TileCfg* cb = col_for(lq);
    const TileCfg* r =
        choice.row_loge >= 0 ? find_tile(STEP_ROW, lp, choice.row_loge, lr_of(choice.row_logr), choice.row_logc) : nullptr;
    if (!r) r = find_tile(STEP_ROW, lp, 4, 4, row_c[lp]);
    if (!ca || !cb || !r || cb->logc > lp || ca->logc > lq + lp || r->logc > lr + lq) {
      set_err(err, "no three-pass tiles instantiated for log2 N = %lld with first column DFTs of 2^%lld", logn, lr);
      return false;
    }
    long long chunk = choice.chunk > 0 ? choice.chunk : std::max(1LL, (1LL << 27) / n);
    chunk = std::min(chunk, batch);
    p.scratch_elems = chunk * n;
    // pipelined = 2: the bulk-load variants (the default); other values run the plain tiles
    PlanChoice pc = choice;
    if (three_default) pc.pipe = 2;
    if (pc.pipe != 2) pc.pipe = 0;
    for (long long b0 = 0; b0 < batch; b0 += chunk) {
      const long long cnt = std::min(chunk, batch - b0);
      Step a{STEP_COL, ca->logm, ca->loge, ca->logr, ca->logc, cnt << (logn - lr - ca->logc), BUF_IN, BUF_OUT,
             b0 * n, cnt * n, b0 * n, cnt * n, cnt, logn};
      Step b{STEP_COL, cb->logm, cb->loge, cb->logr, cb->logc, (cnt << lr) << (lp - cb->logc), BUF_OUT, BUF_SCRATCH,
             b0 * n, cnt * n, 0, cnt * n, cnt << lr, lq + lp};
      Step c{STEP_ROW, r->logm, r->loge, r->logr, r->logc, cnt << (logn - lp - r->logc), BUF_SCRATCH, BUF_OUT,
             0, cnt * n, b0 * n, cnt * n, cnt, logn};
      b.ologr = lr;
      a.pipe = use_pipe(pc, ca);
      b.pipe = use_pipe(pc, cb);
      c.pipe = use_pipe(pc, r);
      p.steps.push_back(a);
      p.steps.push_back(b);
      p.steps.push_back(c);
    }
    p.hbm_passes = 3;
    *out = p;
    return true;
  }

  if (mode == 1 && !tc && (choice.single_cluster > 0 || cluster_default)) {
    // one transform per thread-block cluster (cluster_core.cuh)
    const TileCfg* c =
        cluster_default
            ? default_cluster(logn)
            : find_tile(STEP_SINGLE, logn, choice.single_loge >= 0 ? choice.single_loge : 4, 4, 0, 0, 0,
                        choice.single_cluster, choice.logn2);
    if (!c) {
      set_err(err, "no cluster tile instantiated for log2 n = %lld with 2^%lld CTAs per transform", logn,
              choice.single_cluster);
      return false;
    }
    Step s{STEP_SINGLE, logn, c->loge, c->logr, 0, batch << c->cluster, BUF_IN, BUF_OUT, 0, total, 0, total, batch, logn};
    s.cluster = c->cluster;
    s.csplit = c->csplit;
    p.steps.push_back(s);
    p.hbm_passes = 1;
    *out = p;
    return true;
  }

  if (mode == 1) {
    if (logn > kSingleMaxLog) {
      set_err(err, "single-kernel plan needs log2 n <= %lld (got %lld)", kSingleMaxLog, logn);
      return false;
    }
    const TileCfg* c = nullptr;
    if (tc)
      c = find_tc(STEP_SINGLE, logn, choice.single_logc);
    else if (choice.single_loge >= 0)
      c = find_tile(STEP_SINGLE, logn, choice.single_loge, lr_of(choice.single_logr), choice.single_logc);
    else
      c = default_single(logn);
    if (!c) {
      set_err(err, "no single-kernel tile instantiated for log2 n = %lld", logn);
      return false;
    }
    // pipelined = 2 with one transform per tile: the persistent bulk-load row
    // tile with N2 = 1 (one row = one whole transform)
    if (!tc && choice.pipe == 2 && c->logc == 0 && find_tile(STEP_ROW, logn, c->loge, c->logr, 0, 2)) {
      Step s{STEP_ROW, logn, c->loge, c->logr, 0, batch, BUF_IN, BUF_OUT, 0, total, 0, total, batch, logn};
      s.pipe = 2;
      p.steps.push_back(s);
      p.hbm_passes = 1;
      *out = p;
      return true;
    }
    const long long per = 1LL << c->logc;
    Step s{STEP_SINGLE, c->logm, c->loge, c->logr, c->logc, (batch + per - 1) / per, BUF_IN, BUF_OUT,
           0, total, 0, total, batch, logn};
    s.pipe = tc ? 0 : use_pipe(choice, c);
    // planner default (measured on a GB300, 1 GiB batches): 2^13 runs the
    // resident radix-32 tile (next transform's bulk copy under this one's
    // passes), 4.5% faster than the plain tile
    if (!tc && choice.mode == 0 && choice.pipe == 0 && logn == 13 && find_tile(STEP_SINGLE, 13, c->loge, c->logr, 0, 3))
      s.pipe = 3;
    s.tc = tc ? 1 : 0;
    p.steps.push_back(s);
    p.hbm_passes = 1;
    *out = p;
    return true;
  }

  // four-step.  Defaults: the autotuner's winners on a GB300 for 1 GiB
  // batches, log2 N -> (log2 N2, column log2 E / log2 C, row log2 E / log2 C,
  // pipelined: 2 = the bulk-load variants where they exist, column / row log2
  // radix); other lengths split N2 = 2^floor(log2 N / 2).
  static const int tuned4[][9] = {
      {15, 7, 4, 5, 4, 3, 0, 4, 4},  {16, 7, 4, 5, 4, 3, 2, 4, 4},  {17, 7, 4, 5, 5, 3, 2, 4, 5},
      {18, 9, 4, 3, 4, 3, 2, 4, 4},  {19, 9, 5, 4, 5, 3, 2, 5, 5},  {20, 10, 5, 3, 5, 3, 2, 5, 5},
      {21, 11, 5, 2, 5, 3, 2, 5, 5}, {22, 11, 5, 2, 4, 2, 2, 5, 4}, {23, 11, 4, 2, 4, 2, 2, 4, 4},
      {24, 12, 5, 2, 5, 2, 0, 4, 4}};
  const int* td = nullptr;
  if (!tc && choice.logn2 < 0 && choice.col_loge < 0 && choice.row_loge < 0)
    for (const auto& t : tuned4)
      if (t[0] == logn) td = t;
  int logn2 = choice.logn2 >= 0 ? choice.logn2 : (td ? td[1] : logn / 2);
  int logn1 = logn - logn2;
  const TileCfg* col = nullptr;
  const TileCfg* row = nullptr;
  if (tc) {
    col = find_tc(STEP_COL, logn2, choice.col_logc);
    row = find_tc(STEP_ROW, logn1, choice.row_logc);
  } else if (td) {
    col = find_tile(STEP_COL, logn2, td[2], td[7], td[3]);
    row = find_tile(STEP_ROW, logn1, td[4], td[8], td[5]);
  } else {
    if (choice.col_loge >= 0)
      col = find_tile(STEP_COL, logn2, choice.col_loge, lr_of(choice.col_logr), choice.col_logc);
    else
      col = default_pass(STEP_COL, logn2, logn1, logn1);
    if (choice.row_loge >= 0)
      row = find_tile(STEP_ROW, logn1, choice.row_loge, lr_of(choice.row_logr), choice.row_logc);
    else
      row = default_pass(STEP_ROW, (int)logn1, std::min((int)logn2, logn1 <= 9 ? 3 : 2), (int)logn2);
  }
  if (!col || !row) {
    set_err(err, "no four-step tiles instantiated for N1 = 2^%lld, N2 = 2^%lld", logn1, logn2);
    return false;
  }
  if (col->logc > logn1 || row->logc > logn2) {
    set_err(err, "four-step chunk wider than the transform (N1 = 2^%lld, N2 = 2^%lld)", logn1, logn2);
    return false;
  }
  long long chunk = choice.chunk > 0 ? choice.chunk : std::max(1LL, (1LL << 27) / n);
  chunk = std::min(chunk, batch);
  p.scratch_elems = chunk * n;
  for (long long b0 = 0; b0 < batch; b0 += chunk) {
    long long cnt = std::min(chunk, batch - b0);
    Step a{STEP_COL, col->logm, col->loge, col->logr, col->logc, cnt << (logn1 - col->logc), BUF_IN, BUF_SCRATCH,
           b0 * n, cnt * n, 0, cnt * n, cnt, logn};
    Step b{STEP_ROW, row->logm, row->loge, row->logr, row->logc, cnt << (logn2 - row->logc), BUF_SCRATCH, BUF_OUT,
           0, cnt * n, b0 * n, cnt * n, cnt, logn};
    PlanChoice pc = choice;
    if (td && choice.pipe == 0) pc.pipe = td[6];
    a.pipe = tc ? 0 : use_pipe(pc, col);
    b.pipe = tc ? 0 : use_pipe(pc, row);
    a.tc = b.tc = tc ? 1 : 0;
    p.steps.push_back(a);
    p.steps.push_back(b);
  }
  p.hbm_passes = 2;
  *out = p;
  return true;
}

bool make_plan2d(long long xdim, long long ydim, long long batch, const PlanChoice& choice, Plan1D* out,
                 std::string* err) {
  const int logx = ilog2_exact(xdim), logy = ilog2_exact(ydim);
  if (logx < 0 || logy < 0) {
    set_err(err, "2D dimensions must be powers of two (got %lld x %lld)", xdim, ydim);
    return false;
  }
  if (logy > kColumnMaxLog || logx + logy > kPlan2dMaxLog) {
    set_err(err, "2D transform needs ydim <= 2^12 and xdim * ydim <= 2^26 (got 2^%lld rows, 2^%lld points)", logy,
            logx + logy);
    return false;
  }
  if (choice.split != 0) {
    set_err(err, "2D transforms run in FP32 (split precision %lld requested)", choice.split);
    return false;
  }
  if (batch < 1) {
    set_err(err, "batch must be >= 1 (got %lld)", batch);
    return false;
  }
  if (batch > ((1LL << kMaxTotalLog) >> (logx + logy))) {
    set_err(err, "xdim * ydim * batch must be at most 2^%lld elements (got batch %lld)", (long long)kMaxTotalLog,
            batch);
    return false;
  }
  Plan1D p;
  if (!make_plan(xdim, ydim * batch, choice, &p, err)) return false;  // the row FFTs
  if (logy > 0) {
    const TileCfg* col = nullptr;
    for (const TileCfg& c : tile_configs())
      if (c.kind == STEP_COLUMN && c.logm == logy && c.logc <= logx && (!col || c.logc > col->logc)) col = &c;
    if (!col) {
      set_err(err, "no column tile instantiated for ydim = 2^%lld", logy);
      return false;
    }
    const long long total = xdim * ydim * batch;
    Step s{STEP_COLUMN, col->logm, col->loge, col->logr, col->logc, batch << (logx - col->logc), BUF_OUT, BUF_OUT,
           0, total, 0, total, batch, logx + logy};
    p.steps.push_back(s);
    p.hbm_passes += 1;
  }
  p.n = xdim * ydim;
  p.batch = batch;
  p.logn = logx + logy;
  p.xdim = xdim;
  p.ydim = ydim;
  *out = p;
  return true;
}

bool make_plan_bluestein(long long n, long long batch, Plan1D* out, std::string* err) {
  if (n < 3 || ilog2_exact(n) >= 0 || n > (1LL << (kBluesteinMaxLogM - 1))) {
    set_err(err, "Bluestein plans take lengths that are not powers of two, 2 < n <= 2^%lld (got %lld)",
            (long long)(kBluesteinMaxLogM - 1), n);
    return false;
  }
  if (batch < 1) {
    set_err(err, "batch must be >= 1 (got %lld)", batch);
    return false;
  }
  if (batch > (1LL << kMaxTotalLog) / n) {
    set_err(err, "n * batch must be at most 2^40 elements (got n = %lld, batch = %lld)", n, batch);
    return false;
  }
  const long long m = bluestein_m(n);
  Plan1D inner;
  const long long chunk = std::min(batch, std::max(1LL, (1LL << 26) / m));
  if (!make_plan(m, chunk, PlanChoice{}, &inner, err)) return false;
  Plan1D p;
  p.n = n;
  p.batch = batch;
  p.logn = 0;
  p.blue_m = m;
  p.blue_chunk = chunk;
  p.scratch_elems = inner.scratch_elems;
  // M <= 2^14: one fused kernel (bluestein_core.cuh); up to 2^22 the
  // three-launch four-step with the chirps folded in; above: pre-multiply, two
  // M-point FFTs, spectrum multiply, post-multiply
  p.hbm_passes = bluestein_fused(m) ? 1 : bluestein_four_step(m) ? 3 : 2 * inner.hbm_passes + 3;
  *out = p;
  return true;
}

bool make_plan_like(const Plan1D& base, long long batch, Plan1D* out, std::string* err) {
  if (base.blue_m > 0) return make_plan_bluestein(base.n, batch, out, err);
  if (base.xdim > 0) return make_plan2d(base.xdim, base.ydim, batch, base.choice, out, err);
  return make_plan(base.n, batch, base.choice, out, err);
}

std::vector<PlanChoice> plan_candidates(long long n, long long batch) {
  std::vector<PlanChoice> out;
  int logn = ilog2_exact(n);
  if (logn < 0 || logn > kMaxLogN) return out;
  out.push_back(PlanChoice{});
  if (logn == 0) return out;
  if (logn <= kSingleMaxLog) {
    for (const TileCfg& c : tile_configs()) {
      if (c.kind != STEP_SINGLE || c.logm != logn || c.tc || c.pipe >= 3 || c.cluster) continue;
      PlanChoice ch;
      ch.mode = 1;
      ch.single_loge = c.loge;
      ch.single_logr = c.logr;
      ch.single_logc = c.logc;
      ch.pipe = c.pipe;
      out.push_back(ch);
      if (!c.pipe && c.logc == 0 && find_tile(STEP_ROW, logn, c.loge, c.logr, 0, 2)) {
        ch.pipe = 2;  // the same tile with bulk loads (persistent row tile, N2 = 1)
        out.push_back(ch);
      }
      for (int rp : {3, 4})  // the same tile resident: next transform's copy under this one's passes
        if (!c.pipe && c.logc == 0 && find_tile(STEP_SINGLE, logn, c.loge, c.logr, 0, rp)) {
          ch.pipe = rp;
          out.push_back(ch);
        }
    }
  }
  for (const TileCfg& c : tile_configs()) {  // one transform per thread-block cluster
    if (c.kind != STEP_SINGLE || c.logm != logn || !c.cluster) continue;
    PlanChoice ch;
    ch.mode = 1;
    ch.single_loge = c.loge;
    ch.single_logc = 0;
    ch.single_cluster = c.cluster;
    ch.logn2 = c.csplit;
    out.push_back(ch);
  }
  for (int lr = 7; lr <= 9; ++lr)
    for (int lq = 7; lq <= 9; ++lq) {
      const int lp = logn - lr - lq;
      if (lp < 7 || lp > 9) continue;
      for (int pipe : {0, 2}) {
        PlanChoice ch;
        ch.mode = 4;
        ch.logn2 = lr;
        ch.logn3 = lq;
        ch.pipe = pipe;
        out.push_back(ch);
      }
    }
  if (logn >= 14) {
    for (int logn2 = 7; logn2 <= 12; ++logn2) {
      int logn1 = logn - logn2;
      if (logn1 < 7 || logn1 > 12) continue;
      for (const TileCfg& c : tile_configs()) {
        if (c.kind != STEP_COL || c.logm != logn2 || c.logc > logn1 || c.pipe || c.tc) continue;
        for (const TileCfg& r : tile_configs()) {
          if (r.kind != STEP_ROW || r.logm != logn1 || r.logc > logn2 || r.pipe || r.tc) continue;
          for (long long chunk : {0LL, 16LL << 20, 128LL << 20}) {
           for (int pipe : {0, 2}) {
            PlanChoice ch;
            ch.mode = 2;
            ch.logn2 = logn2;
            ch.col_loge = c.loge;
            ch.col_logr = c.logr;
            ch.col_logc = c.logc;
            ch.row_loge = r.loge;
            ch.row_logr = r.logr;
            ch.row_logc = r.logc;
            ch.chunk = chunk == 0 ? 0 : std::max(1LL, chunk / n);
            ch.pipe = pipe;
            out.push_back(ch);
           }
          }
        }
      }
    }
  }
  (void)batch;
  return out;
}

std::string Plan1D::describe() const {
  std::string s;
  char buf[512];
  static const char* splits[] = {"fp32", "fp16x2", "bf16x2", "bf16x3"};
  std::snprintf(buf, sizeof buf,
                "{\"n\": %lld, \"batch\": %lld, \"bluestein_m\": %lld, \"xdim\": %lld, \"ydim\": %lld, \"precision\": \"%s\", "
                "\"hbm_passes\": %d, \"launches\": %zu, \"scratch_bytes\": %lld, \"kernels\": [",
                n, batch, blue_m, xdim, ydim, splits[(choice.split >= 0 && choice.split <= 3) ? choice.split : 0], hbm_passes,
                steps.size(), scratch_elems * 8);
  s += buf;
  const char* names[] = {"single", "col", "row", "copy", "unused", "column"};
  // the first two steps (one chunk), and for 2D plans the column step
  std::vector<size_t> idx;
  for (size_t i = 0; i < steps.size() && i < (size_t)(hbm_passes == 3 ? 3 : 2); ++i)
    if (!(xdim > 0 && steps[i].kind == STEP_COLUMN)) idx.push_back(i);
  if (xdim > 0 && !steps.empty() && steps.back().kind == STEP_COLUMN) idx.push_back(steps.size() - 1);
  int shown = 0;
  for (size_t i : idx) {
    const Step& st = steps[i];
    std::snprintf(buf, sizeof buf,
                  "%s{\"kind\": \"%s\", \"logm\": %d, \"loge\": %d, \"logc\": %d, \"tiles\": %lld, \"pipe\": %d, "
                  "\"tc\": %d, \"cluster\": %d, \"csplit\": %d}",
                  shown ? ", " : "", names[st.kind], st.logm, st.loge, st.logc, st.grid, st.pipe, st.tc, st.cluster,
                  st.csplit);
    s += buf;
    ++shown;
  }
  s += "]}";
  return s;
}

}  // namespace estl
