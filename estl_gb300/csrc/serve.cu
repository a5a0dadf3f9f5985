// serve.cu — request serving loop: 1D FFT and FFT-convolution requests of
// mixed lengths, continuous batching, HBM admission budget, latency stats.
//
// The reference has no server: Convolution2D_FFT::convolve (Convolution.h:95)
// and FFT<D>::execute (FFT.h:35) are blocking calls, one request at a time,
// which is the "plain per-request" mode here (max_batch_requests = 1,
// max_inflight_batches = 1).
//
// One device-owner thread runs the loop:
//   * requests wait in a FIFO queue after estl_serve_submit;
//   * whenever a stream slot is free, the thread admits queued requests in
//     arrival order while their device memory fits the budget (requests that
//     could never fit are rejected at submit time);
//   * an admitted batch gets one stream-ordered allocation (cudaMallocAsync),
//     copies its inputs in, runs the convolution kernels (grouped by padded
//     length) and FFT plans (grouped by length and direction), copies the
//     outputs back to the callers' host buffers and frees its memory, all on
//     its stream; a host callback (cudaLaunchHostFunc) marks it complete;
//   * up to max_inflight_batches batches overlap on the device, so requests
//     that arrive while others run are admitted as slots and memory free up.
// Each request's arithmetic depends only on its own lengths, so its result is
// bit-identical alone and inside any batch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "conv_exec.h"
#include "engine.h"

using namespace estl;

namespace {

double now_us() {
  return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

struct Req {
  uint64_t ticket = 0;
  estl_serve_request r{};
  double t_submit = 0, t_admit = 0, t_launch = 0, t_done = 0;
  estl_status status = ESTL_OK;
  size_t bytes = 0;
  int batch_requests = 0;
  bool done = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  bool busy = false;
  // pinned staging for the convolution descriptors of a batch
  ConvRow* pinned_rows = nullptr;
  size_t pinned_rows_cap = 0;
};

struct Batch {
  estl_server_s* srv = nullptr;
  int slot = -1;
  std::vector<Req*> reqs;
  size_t bytes = 0;
  double t_launch = 0;
};

}  // namespace

struct estl_server_s {
  estl_serve_config cfg{};
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;       // loop wake-up: submissions, completions, stop
  std::condition_variable cv_done;  // poll wake-up
  std::deque<Req*> queue;
  std::unordered_map<uint64_t, Req*> reqs;
  std::vector<Slot> slots;
  std::vector<Batch*> completed;  // filled by stream callbacks
  uint64_t next_ticket = 1;
  size_t inflight_bytes = 0;
  bool stop = false;
  estl_serve_stats stats{};
  int device = 0;
};

namespace {

// Device bytes a request needs while in flight.
size_t request_bytes(const estl_serve_request& r) {
  if (r.kind == ESTL_REQ_FFT) {
    const size_t n = (size_t)r.n;
    const bool four_step = ilog2_exact(r.n) > kSingleMaxLog;
    return up256(8 * n) * 2 + (four_step ? up256(8 * n) : 0);
  }
  const long long L = r.signal_len, K = r.filter_len;
  const size_t N = (size_t)1 << conv_logn(L, K);
  const size_t out = (size_t)conv_out_len(L, K, r.flags);
  const bool four_step = conv_logn(L, K) > kSingleMaxLog;
  return up256(4 * L) + up256(4 * K) + up256(4 * out) + 2 * sizeof(ConvRow) + 8 * N + (four_step ? 16 * N : 0) + 1024;
}

estl_status validate(const estl_serve_request& r) {
  if (r.kind == ESTL_REQ_FFT) {
    const int l = ilog2_exact(r.n);
    if (l < 0 || l > kMaxLogN) return fail(ESTL_UNSUPPORTED_SIZE, "FFT request length %lld", (long long)r.n);
    if (r.direction != ESTL_FORWARD && r.direction != ESTL_BACKWARD) return fail(ESTL_INVALID_ARG, "bad direction");
    if (r.flags & ~(3 << kConvSplitShift)) return fail(ESTL_INVALID_ARG, "FFT request flags: only a precision");
    if (!r.in || !r.out) return fail(ESTL_INVALID_ARG, "FFT request needs in and out host buffers");
    return ESTL_OK;
  }
  if (r.kind == ESTL_REQ_CONV) {
    if (r.signal_len < 1 || r.filter_len < 1) return fail(ESTL_INVALID_ARG, "convolution lengths must be >= 1");
    if (conv_logn(r.signal_len, r.filter_len) > kConvMaxLogN)
      return fail(ESTL_UNSUPPORTED_SIZE, "convolution padded length above 2^%d", kConvMaxLogN);
    if (r.flags & ~kConvFlagMask) return fail(ESTL_INVALID_ARG, "bad flags");
    if (!r.in || !r.filter || !r.out) return fail(ESTL_INVALID_ARG, "convolution request needs three host buffers");
    return ESTL_OK;
  }
  return fail(ESTL_INVALID_ARG, "unknown request kind %d", r.kind);
}

void CUDART_CB batch_done_cb(void* user) {
  Batch* b = static_cast<Batch*>(user);
  estl_server_s* s = b->srv;
  const double t = now_us();
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (Req* q : b->reqs) q->t_done = t;
    s->completed.push_back(b);
  }
  s->cv.notify_all();
}

// Enqueues one batch on its slot's stream.  Returns the first error (the
// stream work already queued stays valid; the callback still completes it).
estl_status enqueue_batch(estl_server_s* srv, Batch* b) {
  Slot& sl = srv->slots[b->slot];
  cudaStream_t st = sl.stream;
  // ---- layout of the batch allocation
  std::map<int, std::vector<Req*>> conv_groups;                // flags -> requests
  // (n, direction, split precision) -> requests
  std::map<std::tuple<long long, int, int>, std::vector<Req*>> fft;
  for (Req* q : b->reqs) {
    if (q->r.kind == ESTL_REQ_CONV)
      conv_groups[q->r.flags].push_back(q);
    else
      fft[{q->r.n, q->r.direction, conv_split(q->r.flags)}].push_back(q);
  }
  struct ConvGroup {
    std::vector<Req*> reqs;
    std::vector<ConvReq> creqs;
    ConvLayout L;
    size_t o_sig, o_filt, o_out, o_ws;
    long long sig_elems, filt_elems, out_elems;
    int flags;
  };
  struct FftGroup {
    std::vector<Req*> reqs;
    Plan1D plan;
    size_t o_in, o_out, o_scr;
    float sgn;
  };
  std::vector<ConvGroup> cgs;
  std::vector<FftGroup> fgs;
  size_t off = 0;
  size_t rows_needed = 0;
  for (auto& kv : conv_groups) {
    ConvGroup g;
    g.reqs = kv.second;
    g.flags = kv.first;
    long long so = 0, fo = 0, oo = 0;
    for (Req* q : g.reqs) {
      g.creqs.push_back(ConvReq{q->r.signal_len, q->r.filter_len, so, fo, oo});
      so += q->r.signal_len;
      fo += q->r.filter_len;
      oo += conv_out_len(q->r.signal_len, q->r.filter_len, g.flags);
    }
    std::string err;
    if (!build_conv_layout(g.creqs.data(), (int)g.creqs.size(), g.flags, &g.L, &err))
      return fail(ESTL_INVALID_ARG, "%s", err.c_str());
    g.sig_elems = so;
    g.filt_elems = fo;
    g.out_elems = oo;
    g.o_sig = off;
    off = up256(off + 4 * (size_t)so);
    g.o_filt = off;
    off = up256(off + 4 * (size_t)fo);
    g.o_out = off;
    off = up256(off + 4 * (size_t)oo);
    g.o_ws = off;
    off = up256(off + g.L.workspace_bytes);
    rows_needed += g.L.filt_rows.size() + g.L.sig_rows.size();
    cgs.push_back(std::move(g));
  }
  for (auto& kv : fft) {
    FftGroup g;
    g.reqs = kv.second;
    std::string err;
    const long long n = std::get<0>(kv.first);
    PlanChoice choice;
    choice.split = std::get<2>(kv.first);
    if (!make_plan(n, (long long)g.reqs.size(), choice, &g.plan, &err))
      return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
    const size_t bytes = 8 * (size_t)n * g.reqs.size();
    g.sgn = std::get<1>(kv.first) == ESTL_FORWARD ? 1.f : -1.f;
    g.o_in = off;
    off = up256(off + bytes);
    g.o_out = off;
    off = up256(off + bytes);
    g.o_scr = off;
    off = up256(off + 8 * (size_t)g.plan.scratch_elems);
    fgs.push_back(std::move(g));
  }
  b->bytes = std::max<size_t>(off, 256);
  // ---- descriptors go through pinned staging so that their copy is asynchronous
  if (rows_needed > sl.pinned_rows_cap) {
    if (sl.pinned_rows) cudaFreeHost(sl.pinned_rows);
    sl.pinned_rows = nullptr;
    sl.pinned_rows_cap = 0;
    estl_status rc = check_cuda(cudaMallocHost((void**)&sl.pinned_rows, rows_needed * 2 * sizeof(ConvRow)),
                               "cudaMallocHost(descriptors)");
    if (rc != ESTL_OK) return rc;
    sl.pinned_rows_cap = rows_needed * 2;
  }
  char* d = nullptr;
  estl_status s = check_cuda(cudaMallocAsync((void**)&d, b->bytes, st), "cudaMallocAsync(batch)");
  if (s != ESTL_OK) return s;  // s: first error of the enqueue
  size_t row_pos = 0;
  for (ConvGroup& g : cgs) {
    for (size_t i = 0; i < g.reqs.size(); ++i) {
      const estl_serve_request& r = g.reqs[i]->r;
      cudaMemcpyAsync(d + g.o_sig + 4 * g.creqs[i].sig_off, r.in, 4 * r.signal_len, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(d + g.o_filt + 4 * g.creqs[i].filt_off, r.filter, 4 * r.filter_len, cudaMemcpyHostToDevice, st);
    }
    ConvRow* pr = sl.pinned_rows + row_pos;
    std::memcpy(pr, g.L.filt_rows.data(), g.L.filt_rows.size() * sizeof(ConvRow));
    std::memcpy(pr + g.L.filt_rows.size(), g.L.sig_rows.data(), g.L.sig_rows.size() * sizeof(ConvRow));
    char* ws = d + g.o_ws;
    cudaMemcpyAsync(ws + g.L.off_filt_rows, pr, g.L.filt_rows.size() * sizeof(ConvRow), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(ws + g.L.off_sig_rows, pr + g.L.filt_rows.size(), g.L.sig_rows.size() * sizeof(ConvRow),
                    cudaMemcpyHostToDevice, st);
    row_pos += g.L.filt_rows.size() + g.L.sig_rows.size();
    ConvBuffers cb = conv_buffers(g.L, ws, reinterpret_cast<const float*>(d + g.o_sig), g.sig_elems,
                                  reinterpret_cast<const float*>(d + g.o_filt), g.filt_elems,
                                  reinterpret_cast<float*>(d + g.o_out));
    s = launch_conv(g.L, cb, 3, st);
    if (s != ESTL_OK) break;
    for (size_t i = 0; i < g.reqs.size(); ++i) {
      const estl_serve_request& r = g.reqs[i]->r;
      const long long olen = conv_out_len(r.signal_len, r.filter_len, g.flags);
      cudaMemcpyAsync(r.out, d + g.o_out + 4 * g.creqs[i].out_off, 4 * olen, cudaMemcpyDeviceToHost, st);
    }
  }
  for (FftGroup& g : fgs) {
    if (s != ESTL_OK) break;
    const size_t one = 8 * (size_t)g.plan.n;
    for (size_t i = 0; i < g.reqs.size(); ++i)
      cudaMemcpyAsync(d + g.o_in + i * one, g.reqs[i]->r.in, one, cudaMemcpyHostToDevice, st);
    s = launch_steps(g.plan, reinterpret_cast<const cf32*>(d + g.o_in), reinterpret_cast<cf32*>(d + g.o_out),
                     reinterpret_cast<cf32*>(d + g.o_scr), g.sgn, st);
    if (s != ESTL_OK) break;
    for (size_t i = 0; i < g.reqs.size(); ++i)
      cudaMemcpyAsync(g.reqs[i]->r.out, d + g.o_out + i * one, one, cudaMemcpyDeviceToHost, st);
  }
  cudaFreeAsync(d, st);
  estl_status s2 = check_cuda(cudaGetLastError(), "batch enqueue");
  if (s == ESTL_OK) s = s2;
  return s;
}

void serve_loop(estl_server_s* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    // retire completed batches
    while (!s->completed.empty()) {
      Batch* b = s->completed.back();
      s->completed.pop_back();
      s->slots[b->slot].busy = false;
      for (Req* q : b->reqs) {
        s->inflight_bytes -= q->bytes;
        q->done = true;
        s->stats.completed++;
      }
      delete b;
      s->cv_done.notify_all();
    }
    if (s->stop && s->queue.empty()) {
      bool busy = false;
      for (const Slot& sl : s->slots) busy |= sl.busy;
      if (!busy) break;
    }
    // admit a batch into a free slot
    int free_slot = -1;
    for (size_t i = 0; i < s->slots.size(); ++i)
      if (!s->slots[i].busy) {
        free_slot = (int)i;
        break;
      }
    Batch* b = nullptr;
    if (free_slot >= 0 && !s->queue.empty()) {
      b = new Batch;
      b->srv = s;
      b->slot = free_slot;
      const double t = now_us();
      while (!s->queue.empty() && (int)b->reqs.size() < s->cfg.max_batch_requests) {
        Req* q = s->queue.front();
        if (s->inflight_bytes + q->bytes > s->cfg.hbm_budget_bytes) break;  // wait for memory
        s->queue.pop_front();
        s->inflight_bytes += q->bytes;
        q->t_admit = t;
        b->reqs.push_back(q);
      }
      if (b->reqs.empty()) {
        delete b;
        b = nullptr;
      } else {
        s->slots[free_slot].busy = true;
        s->stats.batches++;
        s->stats.max_inflight_bytes = std::max<uint64_t>(s->stats.max_inflight_bytes, s->inflight_bytes);
        s->stats.max_batch_requests = std::max<int64_t>(s->stats.max_batch_requests, (int64_t)b->reqs.size());
        for (Req* q : b->reqs) q->batch_requests = (int)b->reqs.size();
      }
    }
    if (b) {
      // launch outside the lock: submissions and callbacks keep flowing
      lk.unlock();
      const double t = now_us();
      for (Req* q : b->reqs) q->t_launch = t;
      estl_status st = enqueue_batch(s, b);
      if (st != ESTL_OK)
        for (Req* q : b->reqs) q->status = st;
      cudaLaunchHostFunc(s->slots[b->slot].stream, batch_done_cb, b);
      lk.lock();
      continue;
    }
    s->cv.wait(lk);
  }
}

}  // namespace

extern "C" {

estl_status estl_serve_start(const estl_serve_config* cfg, estl_server* out) {
  if (!cfg || !out) return fail(ESTL_INVALID_ARG, "NULL config or server pointer");
  *out = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  std::unique_ptr<estl_server_s> sv(new estl_server_s);
  sv->cfg = *cfg;
  if (sv->cfg.hbm_budget_bytes == 0) {
    Engine& E = engine();
    sv->cfg.hbm_budget_bytes = E.budget > E.used.load() ? E.budget - E.used.load() : 0;
  }
  if (sv->cfg.max_inflight_batches < 1) sv->cfg.max_inflight_batches = 4;
  if (sv->cfg.max_batch_requests < 1) sv->cfg.max_batch_requests = 256;
  if (sv->cfg.max_queue < 1) sv->cfg.max_queue = 1 << 20;
  sv->device = engine().device;
  sv->slots.resize(sv->cfg.max_inflight_batches);
  for (Slot& sl : sv->slots) {
    s = check_cuda(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (s != ESTL_OK) return s;
  }
  estl_server_s* raw = sv.release();
  raw->th = std::thread(serve_loop, raw);
  *out = raw;
  return ESTL_OK;
}

estl_status estl_serve_submit(estl_server s, const estl_serve_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return fail(ESTL_INVALID_ARG, "NULL argument");
  estl_status st = validate(*r);
  if (st != ESTL_OK) return st;
  std::unique_ptr<Req> q(new Req);
  q->r = *r;
  q->bytes = request_bytes(*r);
  q->t_submit = now_us();
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return fail(ESTL_INVALID_ARG, "server is stopping");
    if (q->bytes > s->cfg.hbm_budget_bytes) {
      s->stats.rejected++;
      return fail(ESTL_ADMISSION_REJECTED, "request needs %zu bytes, above the %zu-byte HBM budget", q->bytes,
                  (size_t)s->cfg.hbm_budget_bytes);
    }
    if ((int64_t)s->queue.size() >= s->cfg.max_queue) {
      s->stats.rejected++;
      return fail(ESTL_ADMISSION_REJECTED, "queue full (%lld requests)", (long long)s->cfg.max_queue);
    }
    q->ticket = s->next_ticket++;
    *ticket = q->ticket;
    s->reqs[q->ticket] = q.get();
    s->queue.push_back(q.release());
    s->stats.submitted++;
  }
  s->cv.notify_all();
  return ESTL_OK;
}

estl_status estl_serve_poll(estl_server s, uint64_t ticket, int timeout_ms, estl_serve_result* res) {
  if (!s) return fail(ESTL_INVALID_ARG, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(ESTL_INVALID_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  Req* q = it->second;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(std::max(0, timeout_ms));
  while (!q->done) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !q->done)
      return fail(ESTL_TIMEOUT, "request %llu not complete after %d ms", (unsigned long long)ticket, timeout_ms);
  }
  if (res) {
    res->status = q->status;
    res->latency_us = q->t_done - q->t_submit;
    res->queue_us = q->t_admit - q->t_submit;
    res->device_us = q->t_done - q->t_launch;
    res->batch_requests = q->batch_requests;
  }
  estl_status st = q->status;
  s->reqs.erase(it);
  delete q;
  if (st != ESTL_OK) return fail(st, "request failed on the device");
  return ESTL_OK;
}

estl_status estl_serve_stats_get(estl_server s, estl_serve_stats* out) {
  if (!s || !out) return fail(ESTL_INVALID_ARG, "NULL argument");
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  out->inflight_bytes = s->inflight_bytes;
  out->queued = (int64_t)s->queue.size();
  return ESTL_OK;
}

estl_status estl_serve_stop(estl_server s) {
  if (!s) return ESTL_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->th.joinable()) s->th.join();
  for (Slot& sl : s->slots) {
    if (sl.stream) {
      cudaStreamSynchronize(sl.stream);
      cudaStreamDestroy(sl.stream);
    }
    if (sl.pinned_rows) cudaFreeHost(sl.pinned_rows);
  }
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
  return ESTL_OK;
}

}  // extern "C"
