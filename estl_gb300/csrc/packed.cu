// packed.cu — uneven batches (packed transforms of mixed lengths, and FFT
// convolutions beside them): the persistent work-queue kernel, its CUDA
// graph, and the C ABI.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "conv_exec.h"
#include "engine.h"
#include "packed_core.cuh"
#include "tuner.h"

namespace estl {

__global__ void __launch_bounds__(kPackedThreads, 3) packed_kernel(PackedArgs a) {
  extern __shared__ float2 estl_packed_smem[];
  __shared__ int slot[2];
  packed_run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_packed_smem), slot);
}

}  // namespace estl

using namespace estl;

struct estl_packed_plan_s {
  PackedLayout layout;
  int direction = ESTL_FORWARD;
  // device workspace
  void* ws = nullptr;
  size_t ws_bytes = 0;
  PackedItem* items = nullptr;
  int* class_list = nullptr;
  long long* offsets = nullptr;
  long long* scratch_off = nullptr;
  int* ncol = nullptr;
  unsigned int* counters = nullptr;  // [0] work counter, [1..] done per transform
  int* error = nullptr;
  cf32* scratch = nullptr;
  size_t counter_bytes = 0;
  int grid = 0;  // persistent grid (CTAs)
  size_t smem = 0;
  // graph (captured per (in, out) pair)
  std::mutex mu;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* g_in = nullptr;
  void* g_out = nullptr;
  const float* g_sig = nullptr;
  const float* g_filt = nullptr;
  float* g_cout = nullptr;
  cudaStream_t cap_stream = nullptr;
  // mixed batches: convolution items of the packed kernel (device tables) ...
  long long nconv = 0;
  PackedConv* convs = nullptr;
  int* conv_class_list = nullptr;
  // ... and the convolutions the convolution engine runs, as a graph branch
  std::vector<ConvReq> conv_engine_reqs;
  ConvLayout conv_layout;
  void* conv_ws = nullptr;  // in ws
  long long conv_sig_elems = 0, conv_filt_elems = 0;
  // floats each convolution array must hold: the largest offset + length over every request
  long long need_sig = 0, need_filt = 0, need_out = 0;
  cudaStream_t conv_stream = nullptr;
  cudaEvent_t conv_fork = nullptr, conv_join = nullptr;
  // test hook (estl_packed_plan_set_test_hook)
  int test_skip_kind = -1;
  unsigned long long test_spin_limit = 0;
  // ESTL_PACKED_BUCKETED: one engine plan per length, branches of the graph
  bool bucketed = false;
  std::vector<PackedBucket> buckets;
  std::vector<long long*> b_xoff;   // device offsets of each bucket (in the workspace)
  std::vector<cf32*> b_scratch;     // dense four-step scratch of each bucket (in the workspace)
  std::vector<cudaStream_t> b_streams;
  std::vector<cudaEvent_t> b_events;  // [0] fork, [1 + k] join of bucket k
  long long b_total = 0;              // extent of the caller's buffers (elements)
};

static size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

// Bucketed mode: every bucket's plan on its own stream, forked from and
// joined back into `st` (parallel branches when captured in a graph).
static estl_status bucketed_enqueue(estl_packed_plan p, const cf32* in, cf32* out, cudaStream_t st) {
  const float sgn = p->direction == ESTL_FORWARD ? 1.f : -1.f;
  estl_status s = check_cuda(cudaEventRecord(p->b_events[0], st), "cudaEventRecord(fork)");
  for (size_t k = 0; k < p->buckets.size() && s == ESTL_OK; ++k) {
    s = check_cuda(cudaStreamWaitEvent(p->b_streams[k], p->b_events[0], 0), "cudaStreamWaitEvent(fork)");
    if (s == ESTL_OK)
      s = launch_steps(p->buckets[k].plan, in, out, p->b_scratch[k], sgn, p->b_streams[k], p->b_xoff[k], p->b_total);
    if (s == ESTL_OK) s = check_cuda(cudaEventRecord(p->b_events[1 + k], p->b_streams[k]), "cudaEventRecord(join)");
    if (s == ESTL_OK) s = check_cuda(cudaStreamWaitEvent(st, p->b_events[1 + k], 0), "cudaStreamWaitEvent(join)");
  }
  return s;
}

struct ConvIO {
  const float* sig;
  const float* filt;
  float* out;
};

static estl_status transforms_enqueue(estl_packed_plan p, const cf32* in, cf32* out, const ConvIO& cio,
                                      cudaStream_t st);

// The whole batch on `st`: the convolution engine's launches (if any) on a
// branch forked from and joined back into `st`, beside the transforms.
static estl_status packed_enqueue(estl_packed_plan p, const cf32* in, cf32* out, const ConvIO& cio,
                                  cudaStream_t st) {
  const bool branch = !p->conv_engine_reqs.empty();
  estl_status s = ESTL_OK;
  if (branch) {
    s = check_cuda(cudaEventRecord(p->conv_fork, st), "cudaEventRecord(fork)");
    if (s == ESTL_OK) s = check_cuda(cudaStreamWaitEvent(p->conv_stream, p->conv_fork, 0), "cudaStreamWaitEvent(fork)");
    if (s == ESTL_OK) {
      ConvBuffers b = conv_buffers(p->conv_layout, p->conv_ws, cio.sig, p->conv_sig_elems, cio.filt,
                                   p->conv_filt_elems, cio.out);
      s = launch_conv(p->conv_layout, b, 3, p->conv_stream);
    }
    if (s == ESTL_OK) s = check_cuda(cudaEventRecord(p->conv_join, p->conv_stream), "cudaEventRecord(join)");
    if (s != ESTL_OK) return s;
  }
  s = p->bucketed ? bucketed_enqueue(p, in, out, st) : transforms_enqueue(p, in, out, cio, st);
  if (s == ESTL_OK && branch) s = check_cuda(cudaStreamWaitEvent(st, p->conv_join, 0), "cudaStreamWaitEvent(join)");
  return s;
}

static estl_status transforms_enqueue(estl_packed_plan p, const cf32* in, cf32* out, const ConvIO& cio,
                                      cudaStream_t st) {
  if (p->layout.launch_begin.empty()) return ESTL_OK;  // every convolution runs on the engine
  Engine& E = engine();
  const PackedLayout& L = p->layout;
  estl_status s = check_cuda(cudaMemsetAsync(p->counters, 0, p->counter_bytes, st), "cudaMemsetAsync(counters)");
  if (s != ESTL_OK) return s;
  for (size_t k = 0; k < L.launch_begin.size(); ++k) {
    PackedArgs a;
    a.items = Ptr<const PackedItem>{p->items, (long long)L.items.size()};
    a.item_base = L.launch_begin[k];
    a.nitems = L.launch_count[k];
    a.class_list = Ptr<const int>{p->class_list, (long long)L.class_list.size()};
    a.offsets = Ptr<const long long>{p->offsets, (long long)L.offsets.size()};
    a.scratch_off = Ptr<const long long>{p->scratch_off, (long long)L.scratch_off.size()};
    a.ncol = Ptr<const int>{p->ncol, (long long)L.ncol.size()};
    a.in = Ptr<const cf32>{in, L.total_elems};
    a.out = Ptr<cf32>{out, L.total_elems};
    a.scratch = Ptr<cf32>{p->scratch, L.scratch_elems};
    a.bank = Ptr<const cf32>{E.bank, kBankSize};
    a.next = p->counters;
    a.done = p->counters + 1;
    a.error = p->error;
    a.sgn = p->direction == ESTL_FORWARD ? 1.f : -1.f;
    a.persistent = L.persistent ? 1 : 0;
    a.skip_kind = p->test_skip_kind;
    a.spin_limit = p->test_spin_limit ? p->test_spin_limit : kPackedSpinLimit;
    a.convs = Ptr<const PackedConv>{p->convs, (long long)L.convs.size()};
    a.conv_class_list = Ptr<const int>{p->conv_class_list, (long long)L.conv_class_list.size()};
    a.csig = Ptr<const float>{cio.sig, L.conv_sig_elems};
    a.cfilt = Ptr<const float>{cio.filt, L.conv_filt_elems};
    a.cout = Ptr<float>{cio.out, L.conv_out_elems};
    const long long grid = L.persistent ? std::min<long long>(p->grid, L.launch_count[k]) : L.launch_count[k];
    if (grid < 1 || grid > INT_MAX) return fail(ESTL_UNSUPPORTED_SIZE, "packed grid of %lld CTAs", grid);
    packed_kernel<<<(unsigned)grid, kPackedThreads, p->smem, st>>>(a);
    s = check_cuda(cudaGetLastError(), "packed_kernel launch");
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}

static void packed_release(estl_packed_plan p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  for (cudaStream_t s : p->b_streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : p->b_events)
    if (e) cudaEventDestroy(e);
  if (p->conv_stream) cudaStreamDestroy(p->conv_stream);
  if (p->conv_fork) cudaEventDestroy(p->conv_fork);
  if (p->conv_join) cudaEventDestroy(p->conv_join);
  dev_free(p->ws, p->ws_bytes);
  delete p;
}

static_assert(sizeof(estl_conv_request) == sizeof(ConvReq), "request layout");

// Plan of a mixed batch (nconv = 0: transforms only).
static estl_status packed_create(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                 const ConvReq* reqs, int64_t nconv, int conv_flags, int mode, estl_packed_plan* plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan pointer");
  *plan = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (direction != ESTL_FORWARD && direction != ESTL_BACKWARD) return fail(ESTL_INVALID_ARG, "bad direction %d", direction);
  if (mode != ESTL_PACKED_PERSISTENT && mode != ESTL_PACKED_PER_SIZE && mode != ESTL_PACKED_BUCKETED)
    return fail(ESTL_INVALID_ARG, "bad mode %d", mode);
  std::unique_ptr<estl_packed_plan_s> p(new estl_packed_plan_s);
  std::string err;
  // every request is validated by the layout, which also splits the
  // convolutions into work items and engine requests
  PackedLayout L;
  if (!build_packed_layout(reinterpret_cast<const long long*>(offsets), reinterpret_cast<const long long*>(sizes),
                           count, mode == ESTL_PACKED_PERSISTENT, &L, &err, reqs, nconv, conv_flags))
    return fail(ESTL_INVALID_ARG, "%s", err.c_str());
  p->direction = direction;
  p->nconv = nconv;
  p->need_sig = L.conv_sig_elems;
  p->need_filt = L.conv_filt_elems;
  p->need_out = L.conv_out_elems;
  // bucketed: every convolution runs the convolution engine's own launches
  if (mode == ESTL_PACKED_BUCKETED)
    p->conv_engine_reqs.assign(reqs, reqs + nconv);
  else
    p->conv_engine_reqs = L.conv_engine;
  if (!p->conv_engine_reqs.empty()) {
    if (p->conv_engine_reqs.size() > (size_t)INT_MAX) return fail(ESTL_INVALID_ARG, "too many convolutions");
    if (!build_conv_layout(p->conv_engine_reqs.data(), (int)p->conv_engine_reqs.size(), conv_flags, &p->conv_layout,
                           &err))
      return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
    conv_extents(p->conv_engine_reqs.data(), (int)p->conv_engine_reqs.size(), &p->conv_sig_elems,
                 &p->conv_filt_elems);
  }
  // the convolution engine's part of the workspace: its rows, spectra, scratch
  auto conv_region = [&](size_t& off) {
    const size_t o = off;
    if (!p->conv_engine_reqs.empty()) off = up256(off + p->conv_layout.workspace_bytes);
    return o;
  };
  auto conv_setup = [&](char* w, size_t o_conv) -> estl_status {
    if (p->conv_engine_reqs.empty()) return ESTL_OK;
    p->conv_ws = w + o_conv;
    char* cw = static_cast<char*>(p->conv_ws);
    const ConvLayout& C = p->conv_layout;
    estl_status r = check_cuda(cudaMemcpy(cw + C.off_filt_rows, C.filt_rows.data(), C.filt_rows.size() * sizeof(ConvRow),
                                          cudaMemcpyHostToDevice),
                               "cudaMemcpy(convolution rows)");
    if (r == ESTL_OK)
      r = check_cuda(cudaMemcpy(cw + C.off_sig_rows, C.sig_rows.data(), C.sig_rows.size() * sizeof(ConvRow),
                                cudaMemcpyHostToDevice),
                     "cudaMemcpy(convolution rows)");
    if (r == ESTL_OK) r = check_cuda(cudaStreamCreateWithFlags(&p->conv_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (r == ESTL_OK) r = check_cuda(cudaEventCreateWithFlags(&p->conv_fork, cudaEventDisableTiming), "cudaEventCreate");
    if (r == ESTL_OK) r = check_cuda(cudaEventCreateWithFlags(&p->conv_join, cudaEventDisableTiming), "cudaEventCreate");
    return r;
  };
  if (mode == ESTL_PACKED_BUCKETED) {
    auto choose = [](long long n, long long c) {
      PlanChoice ch;
      tuner_lookup(n, c, &ch);
      return ch;
    };
    if (count > 0 &&
        !build_packed_buckets(reinterpret_cast<const long long*>(offsets), reinterpret_cast<const long long*>(sizes),
                              count, +choose, &p->buckets, &p->b_total, &err))
      return fail(ESTL_INVALID_ARG, "%s", err.c_str());
    p->bucketed = true;
    // workspace: per bucket its offsets, then its scratch; then the convolution engine's
    size_t off = 0;
    std::vector<size_t> o_x, o_s;
    for (const PackedBucket& b : p->buckets) {
      o_x.push_back(off);
      off = up256(off + b.xoff.size() * sizeof(long long));
      o_s.push_back(off);
      off = up256(off + (size_t)b.plan.scratch_elems * sizeof(cf32));
    }
    const size_t o_conv = conv_region(off);
    p->ws_bytes = std::max<size_t>(off, 256);
    s = dev_alloc(&p->ws, p->ws_bytes, "bucketed packed plan workspace");
    if (s != ESTL_OK) return s;
    char* w = static_cast<char*>(p->ws);
    for (size_t k = 0; k < p->buckets.size() && s == ESTL_OK; ++k) {
      p->b_xoff.push_back(reinterpret_cast<long long*>(w + o_x[k]));
      p->b_scratch.push_back(reinterpret_cast<cf32*>(w + o_s[k]));
      s = check_cuda(cudaMemcpy(p->b_xoff[k], p->buckets[k].xoff.data(), p->buckets[k].xoff.size() * sizeof(long long),
                                cudaMemcpyHostToDevice),
                     "cudaMemcpy(bucket offsets)");
      if (s == ESTL_OK) s = prepare_steps(p->buckets[k].plan);
      cudaStream_t bs = nullptr;
      if (s == ESTL_OK) s = check_cuda(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking), "cudaStreamCreate");
      p->b_streams.push_back(bs);
    }
    for (size_t k = 0; k <= p->buckets.size() && s == ESTL_OK; ++k) {
      cudaEvent_t e = nullptr;
      s = check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
      p->b_events.push_back(e);
    }
    if (s == ESTL_OK) s = conv_setup(w, o_conv);
    if (s == ESTL_OK)
      s = check_cuda(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (s != ESTL_OK) {
      packed_release(p.release());
      return s;
    }
    *plan = p.release();
    return ESTL_OK;
  }
  p->layout = std::move(L);
  const PackedLayout& PL = p->layout;
  // workspace: items | class list | offsets | scratch offsets | ncol | counters | error | scratch |
  //            convolution items | their class list | the convolution engine's
  size_t off = 0;
  const size_t o_items = off;
  off = up256(off + std::max<size_t>(PL.items.size(), 1) * sizeof(PackedItem));
  const size_t o_cls = off;
  off = up256(off + std::max<size_t>(PL.class_list.size(), 1) * sizeof(int));
  const size_t o_off = off;
  off = up256(off + PL.offsets.size() * sizeof(long long));
  const size_t o_soff = off;
  off = up256(off + PL.scratch_off.size() * sizeof(long long));
  const size_t o_ncol = off;
  off = up256(off + PL.ncol.size() * sizeof(int));
  const size_t o_cnt = off;
  p->counter_bytes = (1 + PL.offsets.size()) * sizeof(unsigned int);
  off = up256(off + p->counter_bytes);
  const size_t o_err = off;
  off = up256(off + sizeof(int));
  const size_t o_scr = off;
  off = up256(off + (size_t)PL.scratch_elems * sizeof(cf32));
  const size_t o_convs = off;
  off = up256(off + PL.convs.size() * sizeof(PackedConv));
  const size_t o_ccls = off;
  off = up256(off + PL.conv_class_list.size() * sizeof(int));
  const size_t o_conv = conv_region(off);
  p->ws_bytes = off;
  s = dev_alloc(&p->ws, p->ws_bytes, "packed plan workspace");
  if (s != ESTL_OK) return s;
  char* w = static_cast<char*>(p->ws);
  p->items = reinterpret_cast<PackedItem*>(w + o_items);
  p->class_list = reinterpret_cast<int*>(w + o_cls);
  p->offsets = reinterpret_cast<long long*>(w + o_off);
  p->scratch_off = reinterpret_cast<long long*>(w + o_soff);
  p->ncol = reinterpret_cast<int*>(w + o_ncol);
  p->counters = reinterpret_cast<unsigned int*>(w + o_cnt);
  p->error = reinterpret_cast<int*>(w + o_err);
  p->scratch = reinterpret_cast<cf32*>(w + o_scr);
  p->convs = reinterpret_cast<PackedConv*>(w + o_convs);
  p->conv_class_list = reinterpret_cast<int*>(w + o_ccls);
  struct Up {
    void* dst;
    const void* src;
    size_t bytes;
  } ups[] = {{p->items, PL.items.data(), PL.items.size() * sizeof(PackedItem)},
             {p->class_list, PL.class_list.data(), PL.class_list.size() * sizeof(int)},
             {p->offsets, PL.offsets.data(), PL.offsets.size() * sizeof(long long)},
             {p->scratch_off, PL.scratch_off.data(), PL.scratch_off.size() * sizeof(long long)},
             {p->ncol, PL.ncol.data(), PL.ncol.size() * sizeof(int)},
             {p->convs, PL.convs.data(), PL.convs.size() * sizeof(PackedConv)},
             {p->conv_class_list, PL.conv_class_list.data(), PL.conv_class_list.size() * sizeof(int)}};
  for (const Up& u : ups) {
    if (!u.bytes) continue;
    s = check_cuda(cudaMemcpy(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice), "cudaMemcpy(packed tables)");
    if (s != ESTL_OK) {
      packed_release(p.release());
      return s;
    }
  }
  cudaMemset(p->error, 0, sizeof(int));
  p->smem = (size_t)kPackedSmemElems * sizeof(cf32);
  s = check_cuda(cudaFuncSetAttribute(packed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem),
                 "cudaFuncSetAttribute(packed)");
  int per_sm = 0;
  if (s == ESTL_OK)
    s = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, packed_kernel, kPackedThreads, p->smem),
                   "occupancy");
  if (s == ESTL_OK) s = conv_setup(w, o_conv);
  if (s == ESTL_OK)
    s = check_cuda(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (s != ESTL_OK) {
    packed_release(p.release());
    return s;
  }
  p->grid = std::max(1, per_sm) * engine().num_sms;
  *plan = p.release();
  return ESTL_OK;
}

// Replays the plan's graph, captured again when a buffer changes.
static estl_status packed_run(estl_packed_plan p, const void* d_in, void* d_out, const ConvIO& cio, void* stream) {
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  std::lock_guard<std::mutex> g(p->mu);
  if (!p->exec || p->g_in != d_in || p->g_out != d_out || p->g_sig != cio.sig || p->g_filt != cio.filt ||
      p->g_cout != cio.out) {
    // capture the launch sequence once per set of buffers
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
    s = check_cuda(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    if (s != ESTL_OK) return s;
    estl_status s2 = packed_enqueue(p, static_cast<const cf32*>(d_in), static_cast<cf32*>(d_out), cio, p->cap_stream);
    s = check_cuda(cudaStreamEndCapture(p->cap_stream, &p->graph), "cudaStreamEndCapture");
    if (s2 != ESTL_OK) return s2;
    if (s != ESTL_OK) return s;
    s = check_cuda(cudaGraphInstantiate(&p->exec, p->graph, 0), "cudaGraphInstantiate");
    if (s != ESTL_OK) return s;
    p->g_in = d_in;
    p->g_out = d_out;
    p->g_sig = cio.sig;
    p->g_filt = cio.filt;
    p->g_cout = cio.out;
  }
  return check_cuda(cudaGraphLaunch(p->exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

static bool has_transforms(estl_packed_plan p) {
  return p->bucketed ? !p->buckets.empty() : !p->layout.offsets.empty();
}

extern "C" {

estl_status estl_packed_plan_create(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                    int mode, estl_packed_plan* plan) {
  if (count < 1) {
    if (plan) *plan = nullptr;
    return fail(ESTL_INVALID_ARG, "need at least one transform");
  }
  return packed_create(offsets, sizes, count, direction, nullptr, 0, 0, mode, plan);
}

estl_status estl_packed_mixed_plan_create(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                          const estl_conv_request* reqs, int64_t nconv, int conv_flags, int mode,
                                          estl_packed_plan* plan) {
  return packed_create(offsets, sizes, count, direction, reinterpret_cast<const ConvReq*>(reqs), nconv, conv_flags,
                       mode, plan);
}

estl_status estl_packed_execute(estl_packed_plan p, const void* d_in, void* d_out, void* stream) {
  if (!p || !d_in || !d_out) return fail(ESTL_INVALID_ARG, "NULL plan or buffer");
  if (p->nconv) return fail(ESTL_INVALID_ARG, "the plan has convolutions: run it with estl_packed_mixed_execute");
  if (d_in == d_out) return fail(ESTL_INVALID_ARG, "in-place execution is not supported");
  if (((uintptr_t)d_in & 7) || ((uintptr_t)d_out & 7)) return fail(ESTL_INVALID_ARG, "buffers must be 8-byte aligned");
  return packed_run(p, d_in, d_out, ConvIO{nullptr, nullptr, nullptr}, stream);
}

estl_status estl_packed_mixed_execute(estl_packed_plan p, const void* d_in, void* d_out, const float* d_signals,
                                      const float* d_filters, float* d_conv_out, void* stream) {
  if (!p) return fail(ESTL_INVALID_ARG, "NULL plan");
  if (has_transforms(p)) {
    if (!d_in || !d_out) return fail(ESTL_INVALID_ARG, "NULL transform buffer");
    if (d_in == d_out) return fail(ESTL_INVALID_ARG, "in-place execution is not supported");
    if (((uintptr_t)d_in & 7) || ((uintptr_t)d_out & 7))
      return fail(ESTL_INVALID_ARG, "transform buffers must be 8-byte aligned");
  }
  if (p->nconv) {
    if (!d_signals || !d_filters || !d_conv_out) return fail(ESTL_INVALID_ARG, "NULL convolution buffer");
    if (((uintptr_t)d_signals | (uintptr_t)d_filters | (uintptr_t)d_conv_out) & 3)
      return fail(ESTL_INVALID_ARG, "signal, filter and output buffers must be 4-byte aligned");
  }
  return packed_run(p, d_in, d_out, ConvIO{d_signals, d_filters, d_conv_out}, stream);
}

estl_status estl_packed_check(estl_packed_plan p) {
  if (!p) return fail(ESTL_INVALID_ARG, "NULL plan");
  estl_status s = check_cuda(cudaDeviceSynchronize(), "packed execute");
  if (s != ESTL_OK) return s;
  if (p->bucketed) return take_bulk_wait_error();
  int e = 0;
  s = check_cuda(cudaMemcpy(&e, p->error, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy(error flag)");
  if (s != ESTL_OK) return s;
  if (e) {
    cudaMemset(p->error, 0, sizeof(int));
    return fail(ESTL_TIMEOUT, "a row item gave up waiting for its column items");
  }
  return ESTL_OK;
}

estl_status estl_packed_plan_set_test_hook(estl_packed_plan p, int skip_column_items, uint64_t spin_limit) {
  if (!p) return fail(ESTL_INVALID_ARG, "NULL plan");
  if (spin_limit > kPackedSpinLimit) return fail(ESTL_INVALID_ARG, "spin limit above the default %llu", kPackedSpinLimit);
  std::lock_guard<std::mutex> g(p->mu);
  p->test_skip_kind = skip_column_items ? PK_COL : -1;
  p->test_spin_limit = spin_limit;
  // the kernel arguments live in the captured graph: capture again
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  return ESTL_OK;
}

estl_status estl_packed_plan_describe(estl_packed_plan p, char* buf, size_t len) {
  if (!p || !buf || !len) return fail(ESTL_INVALID_ARG, "NULL plan or buffer");
  if (p->bucketed) {
    std::string d = "{\"mode\": \"bucketed\", \"buckets\": [";
    long long elems = 0, launches = 0;
    double flops = 0;
    for (size_t k = 0; k < p->buckets.size(); ++k) {
      const PackedBucket& b = p->buckets[k];
      const long long c = (long long)b.xoff.size();
      elems += c << b.logn;
      flops += 5.0 * (double)(c << b.logn) * b.logn;
      launches += (long long)b.plan.steps.size();
      char e[160];
      const Step& s0 = b.plan.steps.front();
      std::snprintf(e, sizeof e, "%s{\"logn\": %d, \"count\": %lld, \"passes\": %d, \"launches\": %zu, \"cluster\": %d, \"pipe\": %d}",
                    k ? ", " : "", b.logn, c, b.plan.hbm_passes, b.plan.steps.size(), s0.cluster, s0.pipe);
      d += e;
    }
    size_t ntf = 0;
    for (const PackedBucket& b : p->buckets) ntf += b.xoff.size();
    char tail[640];
    std::snprintf(tail, sizeof tail,
                  "], \"transforms\": %zu, \"launches\": %lld, \"elements\": %lld, \"flops\": %.6g, "
                  "\"convolutions\": %lld, \"conv_items\": 0, \"conv_engine\": %zu, \"conv_launches\": %zu, "
                  "\"conv_signal_floats\": %lld, \"conv_filter_floats\": %lld, \"conv_out_floats\": %lld}",
                  ntf, launches + (long long)p->conv_layout.launches.size(), elems, flops, p->nconv,
                  p->conv_engine_reqs.size(), p->conv_layout.launches.size(), p->need_sig, p->need_filt, p->need_out);
    d += tail;
    if (d.size() + 1 > len) return fail(ESTL_INVALID_ARG, "describe buffer of %zu bytes is too small", len);
    std::snprintf(buf, len, "%s", d.c_str());
    return ESTL_OK;
  }
  const PackedLayout& L = p->layout;
  const int n = std::snprintf(
      buf, len,
      "{\"transforms\": %zu, \"items\": %zu, \"launches\": %zu, \"persistent\": %s, \"grid\": %d, "
      "\"elements\": %lld, \"flops\": %.6g, \"scratch_bytes\": %lld, \"smem_bytes\": %zu, \"convolutions\": %lld, "
      "\"conv_items\": %zu, \"conv_engine\": %zu, \"conv_launches\": %zu, \"conv_flops\": %.6g, "
      "\"conv_signal_floats\": %lld, \"conv_filter_floats\": %lld, \"conv_out_floats\": %lld}",
      L.offsets.size(), L.items.size(), L.launch_begin.size() + p->conv_layout.launches.size(),
      L.persistent ? "true" : "false", L.persistent ? p->grid : 0, L.elements, L.flops, L.scratch_elems * 8, p->smem,
      p->nconv, L.convs.size(), p->conv_engine_reqs.size(), p->conv_layout.launches.size(), L.conv_flops, p->need_sig,
      p->need_filt, p->need_out);
  if (n < 0 || (size_t)n >= len) return fail(ESTL_INVALID_ARG, "describe buffer of %zu bytes is too small", len);
  return ESTL_OK;
}

estl_status estl_packed_plan_destroy(estl_packed_plan p) {
  if (!p) return ESTL_OK;
  cudaDeviceSynchronize();
  packed_release(p);
  return ESTL_OK;
}

// One call: plan (persistent mode), execute on `stream`, wait for it, check
// the dependency waits, release the plan.
estl_status estl_execute_packed(const int64_t* offsets, const int64_t* sizes, int64_t count, int direction,
                                const void* d_in, void* d_out, void* stream) {
  estl_packed_plan p = nullptr;
  estl_status s = estl_packed_plan_create(offsets, sizes, count, direction, ESTL_PACKED_PERSISTENT, &p);
  if (s != ESTL_OK) return s;
  s = estl_packed_execute(p, d_in, d_out, stream);
  if (s == ESTL_OK) s = check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
  if (s == ESTL_OK) s = estl_packed_check(p);
  const std::string msg = s == ESTL_OK ? std::string() : std::string(estl_last_error());
  estl_packed_plan_destroy(p);
  if (s != ESTL_OK) return fail(s, "%s", msg.c_str());
  return ESTL_OK;
}

}  // extern "C"
