// emu.cpp — host emulator of the tile FFT kernels (test infrastructure).
//
// Runs the planner's launch list (estl_gb300/csrc/planner.cpp) through the
// same kernel bodies the GPU runs (estl_gb300/csrc/fft_core.cuh, compiled with
// ESTL_EMU): every emulated GPU thread is a host thread, __syncthreads is a
// std::barrier, and every global / shared / twiddle access is bounds checked.
// A CPU test can therefore prove that a kernel configuration stays in bounds
// and computes the right transform before it is launched on a GPU.
#include <ucontext.h>

#include <cmath>
#include <condition_variable>
#include <functional>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "bluestein_core.cuh"
#include "conv_plan.h"
#include "fft_core.cuh"
#include "packed_core.cuh"
#include "bulk_core.cuh"
#include "conv2d_core.cuh"
#include "estl_cuda.h"
#include "resident_core.cuh"
#include "cluster_core.cuh"
#include "planner.h"

using namespace estl;

namespace {
std::mutex g_msg_mu;
std::string g_msg;

struct EmuFault : std::runtime_error {
  using std::runtime_error::runtime_error;
};
}  // namespace

void estl_emu_sync();

void estl_emu_fail(const char* what, long long idx, long long n) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: index %lld outside [0, %lld)", what, idx, n);
  {
    std::lock_guard<std::mutex> g(g_msg_mu);
    if (g_msg.empty()) g_msg = buf;
  }
  throw EmuFault(buf);
}

namespace {

using RunFn = void (*)(const TileArgs&, long long, int, cf32*);
struct EmuKernel {
  int kind, logm, loge, logr, logc, nt;
  long long smem;
  RunFn fn;
  int pipe;
  int tc;
  int cluster, csplit;  // cluster tiles: log2 CTAs per cluster, log2 column DFT length
};

template <class K>
EmuKernel mk(int kind, int m, int e, int r, int c, int pipe = 0, int tc = 0) {
  return EmuKernel{kind, m, e, r, c, K::NT, K::SMEM_ELEMS, &K::run, pipe, tc, cluster_of<K>::log_cluster,
                   cluster_of<K>::log_split};
}

const std::vector<EmuKernel>& emu_kernels() {
  static const std::vector<EmuKernel> v = [] {
    std::vector<EmuKernel> k;
#define ESTL_X_SINGLE(M, E, R, C) k.push_back(mk<SingleKernel<M, E, R, C>>(STEP_SINGLE, M, E, R, C));
#define ESTL_X_COL(M, E, R, C) k.push_back(mk<ColKernel<M, E, R, C>>(STEP_COL, M, E, R, C));
#define ESTL_X_ROW(M, E, R, C) k.push_back(mk<RowKernel<M, E, R, C>>(STEP_ROW, M, E, R, C));
#define ESTL_X_BULK_ROW(M, E, R, C) k.push_back(mk<BulkRowKernel<M, E, R, C>>(STEP_ROW, M, E, R, C, 2));
#define ESTL_X_BULK_COL(M, E, R, C) k.push_back(mk<BulkColKernel<M, E, R, C>>(STEP_COL, M, E, R, C, 2));
#define ESTL_X_RES(M, E, R, H) k.push_back(mk<ResKernel<M, E, R, H>>(STEP_SINGLE, M, E, R, 0, 2 + H));
#define ESTL_X_CLUSTER(N, LR, N2, E) k.push_back(mk<ClusterKernel<N, LR, N2, E>>(STEP_SINGLE, N, E, 4, 0));
#define ESTL_X_COLUMN(M, E, C) k.push_back(mk<ColKernel<M, E, 4, C, false, false>>(STEP_COLUMN, M, E, 4, C));
#define ESTL_X_TC_SINGLE(M, C) k.push_back(mk<SingleKernel<M, 4, 4, C, true>>(STEP_SINGLE, M, 4, 4, C, 0, 1));
#define ESTL_X_TC_COL(M, C) k.push_back(mk<ColKernel<M, 4, 4, C, true>>(STEP_COL, M, 4, 4, C, 0, 1));
#define ESTL_X_TC_ROW(M, C) k.push_back(mk<RowKernel<M, 4, 4, C, true>>(STEP_ROW, M, 4, 4, C, 0, 1));
#include "kernel_list.inc"
    return k;
  }();
  return v;
}

const std::vector<cf32>& host_bank() {
  static const std::vector<cf32> b = [] {
    std::vector<cf32> v((size_t)kBankSize);
    for (long long idx = 0; idx < kBankSize; ++idx) {
      long double x;
      if (idx < kBankDirect) {
        if (idx < 2) {
          v[idx] = cf32{1.f, 0.f};
          continue;
        }
        int k = 0;
        while ((2LL << k) <= idx) k++;
        long long j = idx - (1LL << k);
        x = -(long double)j / (long double)(1LL << (k - 1));
      } else {
        long long r = idx - kBankDirect;
        int n = kBankLog + 1 + (int)(r >> kLoLog);
        long long j = r & ((1LL << kLoLog) - 1);
        x = -(long double)j / (long double)(1LL << (n - 1));
      }
      const long double pi = 3.14159265358979323846264338327950288L;
      v[idx] = cf32{(float)cosl(pi * x), (float)sinl(pi * x)};
    }
    return v;
  }();
  return b;
}

// The threads of one emulated CTA (or of the CTAs of one cluster) are fibers
// (ucontext coroutines) on the calling host thread: a barrier is a yield to a
// scheduler that resumes every fiber that is not waiting, so all fibers reach
// each barrier before any passes it.  No OS threads, no futexes.  A round
// runs the fibers in thread order, or in reverse thread order (every odd CTA
// or cluster of a grid): a shared-memory slot read in the same barrier
// interval in which another thread writes it then holds the old value (or the
// NaN poison) in one of the two orders, and the race fails the parity check.
// In the bulk-load kernels thread 0's copies complete at issue and the
// mbarrier waits return at once: thread order then catches a copy that
// overwrites a stage other threads still read, reverse order a read of a
// stage before its copy.
//
// Clusters: __syncthreads releases the fibers of one CTA, a cluster barrier
// those of every CTA of the cluster.  Each CTA runs on its own as far as it
// can (lowest rank first, or highest first in reverse order) before the next
// CTA runs at all, so a read of another CTA's shared memory that is not
// ordered by a cluster barrier sees the poison in one of the two orders.  A
// CTA whose threads wait at different kinds of barrier is reported.
enum FiberState : char { F_RUN = 0, F_AT_CTA = 1, F_AT_CLUSTER = 2, F_DONE = 3 };
struct FiberSched {
  std::vector<ucontext_t> ctx;
  // not value-initialised: pages a fiber never touches are never committed
  std::vector<std::unique_ptr<char[]>> stacks;
  std::vector<char> state;
  std::vector<long long> arrivals;  // cluster barrier arrives of each fiber
  std::vector<long long> waited;    // the phase of each fiber's last wait
  long long completed = 0;          // cluster barrier phases completed
  ucontext_t main;
  int current = 0;
  const std::function<void(int)>* body = nullptr;
};
thread_local FiberSched* tl_sched = nullptr;
constexpr size_t kFiberStack = 256 * 1024;
// shared memory of the CTAs of the emulated cluster (estl_emu_cluster_smem)
thread_local std::vector<cf32*>* tl_cluster_smem = nullptr;
thread_local long long tl_cluster_smem_elems = 0;

void fiber_entry() {
  FiberSched* s = tl_sched;
  const int f = s->current;
  (*s->body)(f);
  s->state[f] = F_DONE;
  // returning resumes uc_link (the scheduler)
}

// Runs ncta * nt fibers; fiber f is thread f % nt of CTA f / nt.  Returns
// false if the fibers deadlocked on mismatched barriers.
bool run_fibers(int nt, const std::function<void(int)>& body, bool reverse, int ncta = 1) {
  static thread_local FiberSched sched;
  FiberSched& s = sched;
  const int total = nt * ncta;
  if ((int)s.stacks.size() < total) {
    s.stacks.resize(total);
    for (auto& st : s.stacks)
      if (!st) st.reset(new char[kFiberStack]);
  }
  s.ctx.assign(total, ucontext_t{});
  s.state.assign(total, F_RUN);
  s.arrivals.assign(total, 0);
  s.waited.assign(total, 0);
  s.completed = 0;
  s.body = &body;
  tl_sched = &s;
  for (int f = 0; f < total; ++f) {
    getcontext(&s.ctx[f]);
    s.ctx[f].uc_stack.ss_sp = s.stacks[f].get();
    s.ctx[f].uc_stack.ss_size = kFiberStack;
    s.ctx[f].uc_link = &s.main;
    makecontext(&s.ctx[f], fiber_entry, 0);
  }
  bool ok = true;
  for (;;) {
    for (int ci = 0; ci < ncta; ++ci) {
      const int cta = reverse ? ncta - 1 - ci : ci;
      for (;;) {  // this CTA until its fibers wait at a cluster barrier or finish
        for (int i = 0; i < nt; ++i) {
          const int f = cta * nt + (reverse ? nt - 1 - i : i);
          if (s.state[f] != F_RUN) continue;
          s.current = f;
          swapcontext(&s.main, &s.ctx[f]);
        }
        int at_cta = 0, other = 0;
        for (int t = 0; t < nt; ++t) {
          const char st = s.state[cta * nt + t];
          if (st == F_AT_CTA) at_cta++;
          else if (st != F_DONE) other++;
        }
        if (at_cta && !other) {
          for (int t = 0; t < nt; ++t)
            if (s.state[cta * nt + t] == F_AT_CTA) s.state[cta * nt + t] = F_RUN;
          continue;
        }
        break;
      }
    }
    int done = 0;
    long long min_arrivals = -1;
    for (int f = 0; f < total; ++f) {
      if (s.state[f] == F_DONE) {
        done++;
        continue;
      }
      if (min_arrivals < 0 || s.arrivals[f] < min_arrivals) min_arrivals = s.arrivals[f];
    }
    if (done == total) break;
    if (min_arrivals > s.completed) {  // every running thread arrived: phases up to min_arrivals complete
      s.completed = min_arrivals;
      bool woke = false;
      for (int f = 0; f < total; ++f)
        if (s.state[f] == F_AT_CLUSTER && s.waited[f] <= s.completed) {
          s.state[f] = F_RUN;
          woke = true;
        }
      if (woke) continue;
    }
    ok = false;  // mismatched barriers: nothing can run
    break;
  }
  tl_sched = nullptr;
  return ok;
}

template <class Fn, class Args>
bool run_generic(int nt, long long smem_elems, Fn fn, const Args& a, long long grid, int ncta = 1) {
  // the device limit on dynamic shared memory per CTA (227 KB on sm_103a)
  if (smem_elems * (long long)sizeof(cf32) > 227LL * 1024) {
    std::lock_guard<std::mutex> g(g_msg_mu);
    if (g_msg.empty()) g_msg = "kernel needs " + std::to_string(smem_elems * sizeof(cf32)) + " bytes of shared memory";
    return false;
  }
  if (ncta < 1 || grid % ncta) {
    std::lock_guard<std::mutex> g(g_msg_mu);
    if (g_msg.empty()) g_msg = "grid is not a whole number of clusters";
    return false;
  }
  // shared memory bases 256-byte aligned, like the device's dynamic shared memory
  const size_t elems = (size_t)std::max<long long>(smem_elems, 1);
  std::vector<std::vector<cf32>> stores(ncta, std::vector<cf32>(elems + 32));
  std::vector<cf32*> bases(ncta);
  for (int r = 0; r < ncta; ++r)
    bases[r] = reinterpret_cast<cf32*>(((uintptr_t)stores[r].data() + 255) & ~(uintptr_t)255);
  const float nan = std::numeric_limits<float>::quiet_NaN();
  bool failed = false;
  tl_cluster_smem = &bases;
  tl_cluster_smem_elems = (long long)elems;
  for (long long cl = 0; cl < grid / ncta && !failed; ++cl) {
    // poison shared memory so that a read of a slot this CTA never wrote
    // shows up as NaN in the output
    for (cf32* b : bases)
      for (size_t e = 0; e < elems; ++e) b[e] = cf32{nan, nan};
    std::function<void(int)> body = [&](int f) {
      const int r = f / nt, tid = f % nt;
      try {
        fn(a, cl * ncta + r, tid, bases[r]);
      } catch (const EmuFault&) {
        failed = true;
      }
    };
    if (!run_fibers(nt, body, (cl & 1) != 0, ncta)) {
      std::lock_guard<std::mutex> g(g_msg_mu);
      if (g_msg.empty()) g_msg = "threads wait at mismatched barriers (deadlock)";
      failed = true;
    }
  }
  tl_cluster_smem = nullptr;
  return !failed;
}

bool run_kernel(const EmuKernel& k, const TileArgs& a, long long grid) {
  return run_generic(k.nt, k.smem, k.fn, a, grid, 1 << k.cluster);
}

}  // namespace

// __syncthreads of an emulated thread: wait for the other threads of its CTA.
void estl_emu_sync() {
  FiberSched* s = tl_sched;
  s->state[s->current] = F_AT_CTA;
  swapcontext(&s->ctx[s->current], &s->main);
}

// Split cluster barrier.  An arrive counts the thread into the cluster's next
// barrier phase; a wait blocks until every thread of the cluster has arrived
// at the phase of the thread's last arrive.  A thread that arrived keeps
// running until its wait, and a wait whose phase has completed returns at
// once, as on the device: work between the two overlaps the other CTAs, and a
// read of another CTA's shared memory before the phase completed sees the
// poison in one of the two scheduling orders.
void estl_emu_cluster_arrive() {
  FiberSched* s = tl_sched;
  s->arrivals[s->current]++;
}
void estl_emu_cluster_wait() {
  FiberSched* s = tl_sched;
  const long long phase = s->arrivals[s->current];  // wait for phase `phase` to complete
  if (phase < 1 || phase <= s->waited[s->current]) estl_emu_fail("cluster wait without an arrive", s->current, 0);
  s->waited[s->current] = phase;
  if (s->completed >= phase) return;
  s->state[s->current] = F_AT_CLUSTER;
  swapcontext(&s->ctx[s->current], &s->main);
}

// Cluster barrier: arrive and wait.
void estl_emu_cluster_sync() {
  estl_emu_cluster_arrive();
  estl_emu_cluster_wait();
}

cf32* estl_emu_cluster_smem(int rank, long long* n) {
  if (!tl_cluster_smem || rank < 0 || rank >= (int)tl_cluster_smem->size()) estl_emu_fail("cluster rank", rank, 0);
  *n = tl_cluster_smem_elems;
  return (*tl_cluster_smem)[rank];
}

namespace {

// ---- convolution kernels ----
using ConvFn = void (*)(const ConvArgs&, long long, int, cf32*);
struct EmuConvKernel {
  int kind, logm, loge, logr, logc, nt;
  long long smem;
  ConvFn fn;
  int tc;
};

template <class K>
EmuConvKernel mkc(int kind, int m, int e, int r, int c, int tc = 0) {
  return EmuConvKernel{kind, m, e, r, c, K::NT, K::SMEM_ELEMS, &K::run, tc};
}

const std::vector<EmuConvKernel>& emu_conv_kernels() {
  static const std::vector<EmuConvKernel> v = [] {
    std::vector<EmuConvKernel> k;
#define ESTL_XC_SINGLE(M, E, R, C)                                      \
  k.push_back(mkc<SpecSingleKernel<M, E, R, C>>(CK_SPEC_SINGLE, M, E, R, C)); \
  k.push_back(mkc<ConvSingleKernel<M, E, R, C>>(CK_CONV_SINGLE, M, E, R, C)); \
  k.push_back(mkc<SpecPairKernel<M, E, R, C>>(CK_SPEC_PAIR, M, E, R, C));     \
  k.push_back(mkc<ConvPairKernel<M, E, R, C>>(CK_CONV_PAIR, M, E, R, C));
#define ESTL_XC_COL(M, E, R, C)                                                       \
  k.push_back(mkc<ConvColKernel<M, E, R, C>>(CK_COL_FILTER, M, E, R, C));               \
  k.push_back(mkc<ConvColKernel<M, E, R, C>>(CK_COL_SIGNAL, M, E, R, C));               \
  k.push_back(mkc<ConvColKernel<M, E, R, C, false, true>>(CK_COL_FILTER_H, M, E, R, C)); \
  k.push_back(mkc<ConvColKernel<M, E, R, C, false, true>>(CK_COL_SIGNAL_H, M, E, R, C));
#define ESTL_XC_ROW(M, E, R, C)                                              \
  k.push_back(mkc<SpecRowKernel<M, E, R, C>>(CK_SPEC_ROW, M, E, R, C));        \
  k.push_back(mkc<ConvMidKernel<M, E, R, C>>(CK_MID, M, E, R, C));             \
  k.push_back(mkc<SpecRowHalfKernel<M, E, R, C>>(CK_SPEC_ROW_H, M, E, R, C));  \
  k.push_back(mkc<ConvMidHalfKernel<M, E, R, C>>(CK_MID_H, M, E, R, C));
#define ESTL_XC_OUT(M, E, R, C)                                          \
  k.push_back(mkc<ConvOutKernel<M, E, R, C>>(CK_OUT, M, E, R, C)); \
  k.push_back(mkc<ConvOutHalfKernel<M, E, R, C>>(CK_OUT_H, M, E, R, C));
#include "conv_list.inc"
#define ESTL_XC_SINGLE(M, E, R, C)                                                                       \
  if constexpr (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog) {                                            \
    k.push_back(mkc<SpecSingleKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(         \
        CK_SPEC_SINGLE, M, E, R, C, 1));                                                                   \
    k.push_back(mkc<ConvSingleKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(         \
        CK_CONV_SINGLE, M, E, R, C, 1));                                                                   \
    k.push_back(mkc<SpecPairKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(           \
        CK_SPEC_PAIR, M, E, R, C, 1));                                                                     \
    k.push_back(mkc<ConvPairKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(           \
        CK_CONV_PAIR, M, E, R, C, 1));                                                                     \
  }
#define ESTL_XC_COL(M, E, R, C)                                                 \
  k.push_back(mkc<ConvColKernel<M, E, R, C, true>>(CK_COL_FILTER, M, E, R, C, 1)); \
  k.push_back(mkc<ConvColKernel<M, E, R, C, true>>(CK_COL_SIGNAL, M, E, R, C, 1));
#define ESTL_XC_ROW(M, E, R, C)                                               \
  k.push_back(mkc<SpecRowKernel<M, E, R, C, true>>(CK_SPEC_ROW, M, E, R, C, 1)); \
  k.push_back(mkc<ConvMidKernel<M, E, R, C, true>>(CK_MID, M, E, R, C, 1));
#define ESTL_XC_OUT(M, E, R, C) k.push_back(mkc<ConvOutKernel<M, E, R, C, true>>(CK_OUT, M, E, R, C, 1));
#include "conv_list.inc"
    return k;
  }();
  return v;
}

void set_err(char* err, int len, const std::string& s) {
  if (err && len > 0) std::snprintf(err, (size_t)len, "%s", s.c_str());
}

PlanChoice choice_from(const int* f) {
  PlanChoice c;
  if (!f) return c;
  c.mode = f[0];
  c.single_loge = f[1];
  c.single_logc = f[2];
  c.logn2 = f[3];
  c.col_loge = f[4];
  c.col_logc = f[5];
  c.row_loge = f[6];
  c.row_logc = f[7];
  c.chunk = f[8];
  c.pipe = f[10];
  c.split = f[11];
  c.logn3 = f[12];
  c.single_logr = f[13];
  c.col_logr = f[14];
  c.row_logr = f[15];
  c.single_cluster = f[16];
  return c;
}

}  // namespace

namespace {
struct EmuC2Kernel {
  int col, logm, loge, logc, nt;
  long long smem;
  void (*fn)(const Conv2dArgs&, long long, int, cf32*);
};

template <class K>
EmuC2Kernel mk_c2(int col, int m, int e, int c) {
  return EmuC2Kernel{col, m, e, c, K::NT, K::SMEM_ELEMS, &K::run};
}

const std::vector<EmuC2Kernel>& emu_c2_kernels() {
  static const std::vector<EmuC2Kernel> v = [] {
    std::vector<EmuC2Kernel> k;
#define ESTL_X_C2ROW(M, E, C) k.push_back(mk_c2<Conv2dRowKernel<M, E, 4, C>>(0, M, E, C));
#define ESTL_X_C2COL(M, E, C) k.push_back(mk_c2<Conv2dColKernel<M, E, 4, C>>(1, M, E, C));
#include "conv2d_list.inc"
    return k;
  }();
  return v;
}

// the tile choice of conv2d.cu: the row tile of the width, the widest column
// tile no wider than the padded width
const EmuC2Kernel* emu_c2_pick(int col, int logm, int logw) {
  const EmuC2Kernel* best = nullptr;
  for (const EmuC2Kernel& d : emu_c2_kernels())
    if (d.col == col && d.logm == logm && (!col || d.logc <= logw) && (!best || d.logc > best->logc)) best = &d;
  return best;
}
}  // namespace

extern "C" {

// Runs the plan for (n, batch) on interleaved complex64 host data.
// choice: 16 ints (PlanChoice fields) or NULL for the planner default.
// sign: -1 forward, +1 backward.  Returns 0 ok, 1 out-of-bounds access,
// 2 plan error, 3 missing kernel.
static int run_plan(const Plan1D& p, int sign, const float* in, float* out, char* err, int errlen,
                    const long long* xoff = nullptr, long long extent = 0);

int emu_plan_run(long long n, long long batch, const int* choice, int sign, const float* in, float* out, char* err,
                 int errlen) {
  Plan1D p;
  std::string e;
  if (!make_plan(n, batch, choice_from(choice), &p, &e)) {
    set_err(err, errlen, e);
    return 2;
  }
  return run_plan(p, sign, in, out, err, errlen);
}

// 2D plan (make_plan2d) of batch arrays of ydim rows by xdim columns.
int emu_plan2d_run(long long xdim, long long ydim, long long batch, int sign, const float* in, float* out, char* err,
                   int errlen) {
  Plan1D p;
  std::string e;
  if (!make_plan2d(xdim, ydim, batch, PlanChoice{}, &p, &e)) {
    set_err(err, errlen, e);
    return 2;
  }
  return run_plan(p, sign, in, out, err, errlen);
}

// Bluestein plan (make_plan_bluestein) of a length that is not a power of
// two: the same element functions as the GPU kernels (bluestein_core.cuh)
// around emulated power-of-two FFT plans.
int emu_bluestein_run(long long n, long long batch, int sign, const float* in, float* out, char* err, int errlen) {
  Plan1D p;
  std::string e;
  if (!make_plan_bluestein(n, batch, &p, &e)) {
    set_err(err, errlen, e);
    return 2;
  }
  const long long M = p.blue_m;
  const float sgn = sign < 0 ? 1.f : -1.f;
  std::vector<cf32> chirp(n), b(M), spec(M);
  for (long long i = 0; i < n; ++i) chirp[i] = bluestein_chirp(i, n);
  for (long long m = 0; m < M; ++m) b[m] = bluestein_kernel_elem(chirp.data(), m, n, M);
  Plan1D one;
  if (!make_plan(M, 1, PlanChoice{}, &one, &e)) {
    set_err(err, errlen, e);
    return 2;
  }
  int rc = run_plan(one, -1, reinterpret_cast<const float*>(b.data()), reinterpret_cast<float*>(spec.data()), err, errlen);
  if (rc) return rc;
  for (cf32& v : spec) v = cf32{v.x / (float)M, v.y / (float)M};
  const cf32* x = reinterpret_cast<const cf32*>(in);
  cf32* y = reinterpret_cast<cf32*>(out);
  if (bluestein_fused(M)) {
    // the fused one-pass kernel of the GPU path, every transform in one launch
    BlueArgs a;
    a.in = Ptr<const cf32>{x, batch * n};
    a.out = Ptr<cf32>{y, batch * n};
    a.chirp = Ptr<const cf32>{chirp.data(), n};
    a.spec = Ptr<const cf32>{spec.data(), M};
    a.bank = Ptr<const cf32>{host_bank().data(), kBankSize};
    a.n = n;
    a.count = batch;
    a.sgn = sgn;
    bool ok = false, found = false;
    auto go = [&](auto kernel_tag) {
      using K = decltype(kernel_tag);
      if (found || (1LL << K::TL::LM) != M) return;
      found = true;
      const long long grid = (batch + K::C - 1) / K::C;
      ok = run_generic(K::NT, K::SMEM_ELEMS,
                       [](const BlueArgs& args, long long cta, int tid, cf32* sm) { K::run(args, cta, tid, sm); }, a,
                       grid);
    };
#define ESTL_BLUE_GO(M_, E_, R_, C_) go(BlueSingleKernel<M_, E_, R_, C_>{});
    ESTL_BLUE_TILES(ESTL_BLUE_GO)
#undef ESTL_BLUE_GO
    if (!found) {
      set_err(err, errlen, "no emulated fused Bluestein kernel");
      return 3;
    }
    if (!ok) {
      std::lock_guard<std::mutex> gl(g_msg_mu);
      set_err(err, errlen, g_msg);
      return 1;
    }
    return 0;
  }
  if (bluestein_four_step(M)) {
    // the three four-step kernels of the GPU path, chunk by chunk
    const int logm = ilog2_exact(M), logn2 = bluestein_logn2(logm), logn1 = logm - logn2;
    std::vector<cf32> spec_p(M);  // Bp[k2*N1 + k1] = Bs[k2 + N2*k1]
    for (long long i = 0; i < M; ++i) spec_p[i] = spec[(i >> logn1) + ((i & ((1LL << logn1) - 1)) << logn2)];
    const float nan = std::numeric_limits<float>::quiet_NaN();
    for (long long b0 = 0; b0 < batch; b0 += p.blue_chunk) {
      const long long c = std::min(p.blue_chunk, batch - b0);
      std::vector<cf32> s1(c * M, cf32{nan, nan}), s2(c * M, cf32{nan, nan});
      BlueArgs a;
      a.in = Ptr<const cf32>{x + b0 * n, c * n};
      a.out = Ptr<cf32>{y + b0 * n, c * n};
      a.chirp = Ptr<const cf32>{chirp.data(), n};
      a.spec = Ptr<const cf32>{spec_p.data(), M};
      a.bank = Ptr<const cf32>{host_bank().data(), kBankSize};
      a.n = n;
      a.count = c;
      a.sgn = sgn;
      a.logm = logm;
      a.s1 = Ptr<cf32>{s1.data(), c * M};
      a.s2 = Ptr<cf32>{s2.data(), c * M};
      bool ok = true;
      int ran = 0;
      auto go = [&](auto kernel_tag, int tile_log, long long units) {
        using K = decltype(kernel_tag);
        if (!ok || K::TL::LM != tile_log) return;
        ++ran;
        ok = run_generic(K::NT, K::SMEM_ELEMS,
                         [](const BlueArgs& args, long long cta, int tid, cf32* sm) { K::run(args, cta, tid, sm); }, a,
                         units / K::C);
      };
#define ESTL_XC_COL(M_, E_, R_, C_) go(BlueColKernel<M_, E_, R_, C_>{}, logn2, c << logn1);
#include "conv_list.inc"
#define ESTL_XC_ROW(M_, E_, R_, C_) go(BlueMidKernel<M_, E_, R_, C_>{}, logn1, c << logn2);
#include "conv_list.inc"
#define ESTL_XC_OUT(M_, E_, R_, C_) go(BlueOutKernel<M_, E_, R_, C_>{}, logn2, c << logn1);
#include "conv_list.inc"
      if (!ok) {
        std::lock_guard<std::mutex> gl(g_msg_mu);
        set_err(err, errlen, g_msg);
        return 1;
      }
      if (ran != 3) {
        set_err(err, errlen, "no emulated four-step Bluestein kernel");
        return 3;
      }
    }
    return 0;
  }
  for (long long b0 = 0; b0 < batch; b0 += p.blue_chunk) {
    const long long c = std::min(p.blue_chunk, batch - b0);
    Plan1D inner;
    if (!make_plan(M, c, PlanChoice{}, &inner, &e)) {
      set_err(err, errlen, e);
      return 2;
    }
    std::vector<cf32> a(c * M), cc(c * M);
    for (long long t = 0; t < c; ++t)
      for (long long m = 0; m < M; ++m) a[t * M + m] = bluestein_pre(x + (b0 + t) * n, chirp.data(), m, n, sgn);
    rc = run_plan(inner, -1, reinterpret_cast<const float*>(a.data()), reinterpret_cast<float*>(cc.data()), err, errlen);
    if (rc) return rc;
    for (long long i = 0; i < c * M; ++i) cc[i] = cmul(cc[i], spec[i % M]);
    rc = run_plan(inner, +1, reinterpret_cast<const float*>(cc.data()), reinterpret_cast<float*>(a.data()), err, errlen);
    if (rc) return rc;
    for (long long t = 0; t < c; ++t)
      for (long long k = 0; k < n; ++k) y[(b0 + t) * n + k] = bluestein_post(a.data() + t * M, chirp.data(), k, sgn);
  }
  return 0;
}

static int run_plan(const Plan1D& p, int sign, const float* in, float* out, char* err, int errlen,
                    const long long* xoff, long long extent) {
  const long long n = p.n, batch = p.batch;
  {
    std::lock_guard<std::mutex> g(g_msg_mu);
    g_msg.clear();
  }
  const long long total = xoff ? extent : n * batch;
  std::vector<cf32> scratch((size_t)std::max<long long>(p.scratch_elems, 1),
                            cf32{std::numeric_limits<float>::quiet_NaN(), 0.f});
  const cf32* cin = reinterpret_cast<const cf32*>(in);
  cf32* cout = reinterpret_cast<cf32*>(out);
  for (const Step& st : p.steps) {
    const cf32* src = st.src == BUF_IN ? cin : (st.src == BUF_SCRATCH ? scratch.data() : cout);
    long long src_cap = st.src == BUF_SCRATCH ? (long long)scratch.size() : total;
    cf32* dst = st.dst == BUF_OUT ? cout : scratch.data();
    long long dst_cap = st.dst == BUF_SCRATCH ? (long long)scratch.size() : total;
    if (st.src_off < 0 || st.src_off + st.src_len > src_cap || st.dst_off < 0 || st.dst_off + st.dst_len > dst_cap) {
      set_err(err, errlen, "step buffer range outside its allocation");
      return 1;
    }
    if (st.kind == STEP_COPY) {
      std::memcpy(dst + st.dst_off, src + st.src_off, (size_t)st.rows * sizeof(cf32));
      continue;
    }
    const EmuKernel* k = nullptr;
    for (const EmuKernel& c : emu_kernels())
      if (c.kind == st.kind && c.logm == st.logm && c.loge == st.loge && c.logr == st.logr && c.logc == st.logc &&
          c.pipe == st.pipe && c.tc == st.tc && c.cluster == st.cluster && c.csplit == st.csplit)
        k = &c;
    if (!k) {
      set_err(err, errlen, "no emulated kernel for a plan step");
      return 3;
    }
    TileArgs a;
    a.in = Ptr<const cf32>{src + st.src_off, st.src_len};
    a.out = Ptr<cf32>{dst + st.dst_off, st.dst_len};
    a.bank = Ptr<const cf32>{host_bank().data(), kBankSize};
    a.rows = st.rows;
    a.logn = st.logn;
    a.logn1 = 0;
    a.sgn = sign < 0 ? 1.f : -1.f;
    a.ologr = st.ologr;
    if (st.ologr) a.sgn = 1.f;  // middle pass of three: its input is conjugated already
    if (xoff) {
      // transforms at the caller's offsets (bucketed uneven batches), as launch_steps
      if (st.src == BUF_OUT || st.ologr || (k->pipe == 2 && st.kind == STEP_COL)) {
        set_err(err, errlen, "a plan step that cannot read transforms through offsets");
        return 2;
      }
      const long long first = st.src == BUF_IN ? st.src_off >> st.logn : st.dst_off >> st.logn;
      if (st.src == BUF_IN) a.in = Ptr<const cf32>{cin, extent};
      if (st.dst == BUF_OUT) a.out = Ptr<cf32>{cout, extent};
      a.xoff = Ptr<const long long>{xoff + first, st.rows};
    }
    // pipelined kernels are grid-stride: emulate one or two CTAs so that every
    // CTA loops over several tiles and uses both tile buffers
    const long long grid = k->pipe ? (st.grid >= 4 ? 2 : 1) : st.grid;
    a.grid = grid;
    a.split = st.tc ? p.choice.split : SPLIT_NONE;
    a.err = nullptr;
    if (!run_kernel(*k, a, grid)) {
      std::lock_guard<std::mutex> g(g_msg_mu);
      set_err(err, errlen, g_msg);
      return 1;
    }
  }
  return 0;
}

// Self-test of the cluster scheduling: each CTA of a cluster of `ncta` writes
// its rank into its own shared memory, synchronises (a cluster barrier when
// cluster_barrier != 0, else only __syncthreads, which does not order another
// CTA's writes) and reads its neighbour's slot.  Returns the number of reads
// that saw the neighbour's value in the worse of the two scheduling orders:
// ncta * nt with the cluster barrier; fewer without it.
int emu_cluster_barrier_selftest(int ncta, int nt, int cluster_barrier) {
  // two clusters: the first runs in forward order, the second in reverse
  std::vector<int> seen(2 * ncta * nt, 0);
  auto body = [&](const int& cb, long long cta, int tid, cf32* sm) {
    const int rank = (int)(cta % ncta);
    sm[tid] = cf32{(float)rank, 0.f};
    if (cb) estl_emu_cluster_sync();
    else estl_emu_sync();
    const int peer = (rank + 1) % ncta;
    const cf32 v = peer_buf(sm, nt, rank, peer)[tid];
    seen[cta * nt + tid] = v.x == (float)peer;
    if (cb) estl_emu_cluster_sync();
    else estl_emu_sync();
  };
  if (!run_generic(nt, nt, body, cluster_barrier, 2LL * ncta, ncta)) return -1;
  int worst = ncta * nt;
  for (int cl = 0; cl < 2; ++cl) {
    int ok = 0;
    for (int i = 0; i < ncta * nt; ++i) ok += seen[cl * ncta * nt + i];
    worst = std::min(worst, ok);
  }
  return worst;
}

// Bucketed uneven batch (build_packed_buckets with the planner defaults):
// every bucket's plan through the transforms' offsets.  Returns 0, 1 (out of
// bounds), 2 (layout error) or 3 (missing kernel).
int emu_packed_bucketed_run(const long long* offsets, const long long* sizes, long long count, int sign,
                            const float* in, float* out, char* err, int errlen) {
  std::vector<PackedBucket> buckets;
  long long extent = 0;
  std::string e;
  if (!build_packed_buckets(offsets, sizes, count, nullptr, &buckets, &extent, &e)) {
    set_err(err, errlen, e);
    return 2;
  }
  for (const PackedBucket& b : buckets) {
    const int rc = run_plan(b.plan, sign, in, out, err, errlen, b.xoff.data(), extent);
    if (rc) return rc;
  }
  return 0;
}

// Plan description (JSON) for (n, batch, choice); returns 0 or 2.
int emu_plan_describe(long long n, long long batch, const int* choice, char* buf, int len) {
  Plan1D p;
  std::string e;
  if (!make_plan(n, batch, choice_from(choice), &p, &e)) {
    set_err(buf, len, e);
    return 2;
  }
  set_err(buf, len, p.describe());
  return 0;
}

// Candidate choices of the autotuner for (n, batch): writes up to max rows
// of 16 ints, returns the number of candidates.
int emu_plan_candidates(long long n, long long batch, int* out, int max) {
  std::vector<PlanChoice> c = plan_candidates(n, batch);
  int k = 0;
  for (const PlanChoice& ch : c) {
    if (k >= max) break;
    int* f = out + 17 * k++;
    f[0] = ch.mode;
    f[1] = ch.single_loge;
    f[2] = ch.single_logc;
    f[3] = ch.logn2;
    f[4] = ch.col_loge;
    f[5] = ch.col_logc;
    f[6] = ch.row_loge;
    f[7] = ch.row_logc;
    f[8] = (int)ch.chunk;
    f[9] = 0;  // formerly the streamed four-step's lag
    f[10] = ch.pipe;
    f[11] = ch.split;
    f[12] = ch.logn3;
    f[13] = ch.single_logr;
    f[14] = ch.col_logr;
    f[15] = ch.row_logr;
    f[16] = ch.single_cluster;
  }
  return (int)c.size();
}

// Batched FFT convolution of real data.  reqs: count x 5 int64
// (signal_len, filter_len, sig_off, filt_off, out_off).  shared: one filter
// (request 0) for all.  Returns 0 ok, 1 out-of-bounds access, 2 layout error,
// 3 missing kernel.
int emu_conv_run(const long long* reqs, int count, int flags, int shared, const float* sig, const float* filt,
                 float* out, char* err, int errlen) {
  ConvLayout L;
  std::string e;
  if (!build_conv_layout(reinterpret_cast<const ConvReq*>(reqs), count, flags, &L, &e, shared != 0)) {
    set_err(err, errlen, e);
    return 2;
  }
  {
    std::lock_guard<std::mutex> g(g_msg_mu);
    g_msg.clear();
  }
  long long se, fe;
  conv_extents(reinterpret_cast<const ConvReq*>(reqs), count, &se, &fe);
  const float nan = std::numeric_limits<float>::quiet_NaN();
  std::vector<cf32> spec((size_t)std::max<long long>(L.spec_elems, 1), cf32{nan, nan});
  std::vector<cf32> s1((size_t)std::max<long long>(L.scratch_elems, 1), cf32{nan, nan});
  std::vector<cf32> s2((size_t)std::max<long long>(L.scratch_elems, 1), cf32{nan, nan});
  for (const ConvLaunch& l : L.launches) {
    const EmuConvKernel* k = nullptr;
    for (const EmuConvKernel& c : emu_conv_kernels())
      if (c.kind == l.kind && c.logm == l.logm && c.loge == l.loge && c.logr == l.logr && c.logc == l.logc &&
          c.tc == l.tc)
        k = &c;
    if (!k) {
      set_err(err, errlen, "no emulated convolution kernel for a launch");
      return 3;
    }
    const long long N = 1LL << l.logn;
    const bool f = ck_is_filter(l.kind);
    const bool four = !ck_is_single(l.kind);
    if (l.s_off + l.row_count * N > (long long)s1.size() && four) {
      set_err(err, errlen, "launch scratch range outside the scratch buffer");
      return 1;
    }
    ConvArgs a;
    const std::vector<ConvRow>& rows = f ? L.filt_rows : L.sig_rows;
    a.rows = Ptr<const ConvRow>{rows.data() + l.row_begin, l.row_count};
    a.nrows = l.row_count;
    a.sig = f ? Ptr<const float>{filt, fe} : Ptr<const float>{sig, se};
    a.spec = Ptr<const cf32>{spec.data(), L.spec_elems};
    a.spec_out = Ptr<cf32>{spec.data(), L.spec_elems};
    a.out = Ptr<float>{out, L.out_elems};
    a.s1 = Ptr<cf32>{s1.data() + (four ? l.s_off : 0), four ? l.row_count * N : 0};
    a.s2 = Ptr<cf32>{s2.data() + (four ? l.s_off : 0), four ? l.row_count * N : 0};
    a.bank = Ptr<const cf32>{host_bank().data(), kBankSize};
    a.logn = l.logn;
    a.split = l.tc ? L.split : SPLIT_NONE;
    a.shared = L.shared;
    if (!run_generic(k->nt, k->smem, k->fn, a, l.grid)) {
      std::lock_guard<std::mutex> g(g_msg_mu);
      set_err(err, errlen, g_msg);
      return 1;
    }
  }
  return 0;
}

// 2D convolution of count images (h rows of w floats) with one filter (kh
// rows of kw floats), the launches of conv2d.cu: filter spectrum (row pass,
// column pass), then row pass, column pass, row pass.  Returns 0 ok, 1
// out-of-bounds access, 2 size error, 3 missing kernel.
int emu_conv2d_run(long long w, long long h, long long kw, long long kh, long long count, int flags,
                   const float* images, const float* filt, float* out, char* err, int errlen) {
  Conv2dGeom g;
  const int compat = (flags & ESTL_CONV_REFERENCE_COMPAT) ? 1 : 0;
  if (count < 1 || !conv2d_geometry(w, h, kw, kh, compat != 0, &g) || !conv2d_supported(g)) {
    set_err(err, errlen, "2D convolution sizes out of range");
    return 2;
  }
  const EmuC2Kernel* row = emu_c2_pick(0, g.logw, g.logw);
  const EmuC2Kernel* col = emu_c2_pick(1, g.logh, g.logw);
  if (!row || !col) {
    set_err(err, errlen, "no emulated 2D convolution tile");
    return 3;
  }
  {
    std::lock_guard<std::mutex> gl(g_msg_mu);
    g_msg.clear();
  }
  const long long pts = 1LL << (g.logw + g.logh);
  const float nan = std::numeric_limits<float>::quiet_NaN();
  std::vector<cf32> spec((size_t)pts, cf32{nan, nan});
  std::vector<cf32> work((size_t)(count * pts), cf32{nan, nan});
  auto launch = [&](const EmuC2Kernel* k, const Conv2dArgs& a) {
    const long long grid = conv2d_grid(k->col != 0, k->logc, a);
    return grid < 1 || run_generic(k->nt, k->smem, k->fn, a, grid);
  };
  Conv2dArgs a = conv2d_filter_args(g, kw, kh, compat, flags & ESTL_CONV_CORRELATE, filt, spec.data(),
                                    host_bank().data(), kBankSize);
  bool ok = launch(row, a);
  a.mode = 1;
  ok = ok && launch(col, a);
  Conv2dArgs b = conv2d_exec_args(g, w, h, count, compat, images, work.data(), spec.data(), out, host_bank().data(),
                                  kBankSize);
  ok = ok && launch(row, b);
  ok = ok && launch(col, b);
  b.mode = 1;
  ok = ok && launch(row, b);
  if (!ok) {
    std::lock_guard<std::mutex> gl(g_msg_mu);
    set_err(err, errlen, g_msg);
    return 1;
  }
  return 0;
}

// Uneven batch: count transforms of lengths sizes[i] at offsets[i] (complex
// elements).  persistent: the work-queue kernel run as one CTA (items in
// queue order); else one CTA per item, launch by launch.  Returns 0 ok,
// 1 out-of-bounds access, 2 layout error, 4 a dependency wait gave up.
int emu_packed_run_launches(const long long* offsets, const long long* sizes, long long count, int persistent,
                            int sign, const float* in, float* out, int skip_columns, char* err, int errlen);

int emu_packed_run(const long long* offsets, const long long* sizes, long long count, int persistent, int sign,
                   const float* in, float* out, char* err, int errlen) {
  return emu_packed_run_launches(offsets, sizes, count, persistent, sign, in, out, 0, err, errlen);
}

// As emu_packed_run, with skip_columns = 1 leaving out every launch that holds
// column items (non-persistent mode): the row items' dependency waits then
// wait for counts that nothing raises, give up after their iteration limit,
// set the error word and skip their work (return 4, output untouched).
static int packed_emulate(const long long* offsets, const long long* sizes, long long count, int persistent,
                          int sign, const float* in, float* out, int skip_columns, const long long* convs,
                          long long nconv, int conv_flags, const float* sig, const float* filt, float* cout,
                          char* err, int errlen);

int emu_packed_run_launches(const long long* offsets, const long long* sizes, long long count, int persistent,
                            int sign, const float* in, float* out, int skip_columns, char* err, int errlen) {
  return packed_emulate(offsets, sizes, count, persistent, sign, in, out, skip_columns, nullptr, 0, 0, nullptr,
                        nullptr, nullptr, err, errlen);
}

// Mixed uneven batch: count transforms (as emu_packed_run) and nconv FFT
// convolutions (5 values each: signal_len, filter_len, signal, filter and
// output offsets in floats, as estl_conv_request), conv_flags as
// estl_conv_execute.  Convolutions of padded length <= 2^12 run as work items
// of the packed kernel, longer ones through the convolution engine's launches
// (as emu_conv_run).  Returns as emu_packed_run.
int emu_packed_mixed_run(const long long* offsets, const long long* sizes, long long count, int persistent, int sign,
                         const float* in, float* out, const long long* convs, long long nconv, int conv_flags,
                         const float* sig, const float* filt, float* cout, char* err, int errlen) {
  return packed_emulate(offsets, sizes, count, persistent, sign, in, out, 0, convs, nconv, conv_flags, sig, filt, cout,
                        err, errlen);
}

static int packed_emulate(const long long* offsets, const long long* sizes, long long count, int persistent,
                          int sign, const float* in, float* out, int skip_columns, const long long* convs,
                          long long nconv, int conv_flags, const float* sig, const float* filt, float* cout,
                          char* err, int errlen) {
  PackedLayout L;
  std::string e;
  if (!build_packed_layout(offsets, sizes, count, persistent != 0, &L, &e,
                           reinterpret_cast<const ConvReq*>(convs), nconv, conv_flags)) {
    set_err(err, errlen, e);
    return 2;
  }
  {
    std::lock_guard<std::mutex> g(g_msg_mu);
    g_msg.clear();
  }
  const float nan = std::numeric_limits<float>::quiet_NaN();
  std::vector<cf32> scratch((size_t)std::max<long long>(L.scratch_elems, 1), cf32{nan, nan});
  std::vector<unsigned int> counters(1 + L.offsets.size(), 0u);
  int error = 0;
  for (size_t k = 0; k < L.launch_begin.size(); ++k) {
    PackedArgs a;
    a.items = Ptr<const PackedItem>{L.items.data(), (long long)L.items.size()};
    a.item_base = L.launch_begin[k];
    a.nitems = L.launch_count[k];
    a.class_list = Ptr<const int>{L.class_list.data(), (long long)L.class_list.size()};
    a.offsets = Ptr<const long long>{L.offsets.data(), (long long)L.offsets.size()};
    a.scratch_off = Ptr<const long long>{L.scratch_off.data(), (long long)L.scratch_off.size()};
    a.ncol = Ptr<const int>{L.ncol.data(), (long long)L.ncol.size()};
    a.in = Ptr<const cf32>{reinterpret_cast<const cf32*>(in), L.total_elems};
    a.out = Ptr<cf32>{reinterpret_cast<cf32*>(out), L.total_elems};
    a.scratch = Ptr<cf32>{scratch.data(), L.scratch_elems};
    a.bank = Ptr<const cf32>{host_bank().data(), kBankSize};
    a.next = counters.data();
    a.done = counters.data() + 1;
    a.error = &error;
    a.sgn = sign < 0 ? 1.f : -1.f;
    a.persistent = persistent ? 1 : 0;
    a.convs = Ptr<const PackedConv>{L.convs.data(), (long long)L.convs.size()};
    a.conv_class_list = Ptr<const int>{L.conv_class_list.data(), (long long)L.conv_class_list.size()};
    a.csig = Ptr<const float>{sig, L.conv_sig_elems};
    a.cfilt = Ptr<const float>{filt, L.conv_filt_elems};
    a.cout = Ptr<float>{cout, L.conv_out_elems};
    counters[0] = 0;
    if (skip_columns && !persistent && a.nitems > 0 && L.items[(size_t)a.item_base].kind == PK_COL) continue;
    int slot[2] = {0, 0};
    auto fn = [&slot](const PackedArgs& args, long long cta, int tid, cf32* sm) { packed_run(args, cta, tid, sm, slot); };
    const long long grid = persistent ? 1 : a.nitems;
    if (!run_generic(kPackedThreads, kPackedSmemElems, fn, a, grid)) {
      std::lock_guard<std::mutex> g(g_msg_mu);
      set_err(err, errlen, g_msg);
      return 1;
    }
  }
  if (error) {
    set_err(err, errlen, "dependency wait gave up");
    return 4;
  }
  if (!L.conv_engine.empty())
    return emu_conv_run(reinterpret_cast<const long long*>(L.conv_engine.data()), (int)L.conv_engine.size(),
                        conv_flags, 0, sig, filt, cout, err, errlen);
  return 0;
}

// Copies the host twiddle bank (kBankSize complex64) into out (if not NULL);
// returns kBankSize.
long long emu_bank(float* out) {
  if (out) std::memcpy(out, host_bank().data(), sizeof(cf32) * (size_t)kBankSize);
  return kBankSize;
}

}  // extern "C"

extern "C" {
// The host emulator's 16-bit conversions (tc_core.cuh), for the conversion
// tests: bf = 1 bfloat16, 0 IEEE binary16; returns the 16-bit pattern.
unsigned emu_to16(float x, int bf) { return estl::to16(x, bf != 0); }
float emu_from16(unsigned h, int bf) { return estl::from16(h, bf != 0); }
}
