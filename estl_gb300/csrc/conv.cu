// conv.cu — FFT convolution: kernel registry, launcher and C ABI.
#include <algorithm>
#include <climits>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "conv_exec.h"

namespace estl {

template <class K>
__global__ void __launch_bounds__(K::NT, K::MINB) conv_kernel(ConvArgs a) {
  extern __shared__ float2 estl_conv_smem[];
  pdl_enter();
  K::run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_conv_smem));
}

namespace {

struct ConvKernelDesc {
  int kind, logm, loge, logr, logc;
  int nthreads, smem_bytes;
  const void* fn;
  bool attr_set;
  int tc;
};

template <class K>
ConvKernelDesc cdesc(int kind, int m, int e, int r, int c, int tc = 0) {
  return ConvKernelDesc{kind, m, e, r, c, K::NT, (int)(K::SMEM_ELEMS * sizeof(cf32)),
                        reinterpret_cast<const void*>(&conv_kernel<K>), false, tc};
}

std::vector<ConvKernelDesc>& conv_table() {
  static std::vector<ConvKernelDesc> t = [] {
    std::vector<ConvKernelDesc> v;
#define ESTL_XC_SINGLE(M, E, R, C)                                          \
  v.push_back(cdesc<SpecSingleKernel<M, E, R, C>>(CK_SPEC_SINGLE, M, E, R, C)); \
  v.push_back(cdesc<ConvSingleKernel<M, E, R, C>>(CK_CONV_SINGLE, M, E, R, C)); \
  v.push_back(cdesc<SpecPairKernel<M, E, R, C>>(CK_SPEC_PAIR, M, E, R, C));     \
  v.push_back(cdesc<ConvPairKernel<M, E, R, C>>(CK_CONV_PAIR, M, E, R, C));
#define ESTL_XC_COL(M, E, R, C)                                                         \
  v.push_back(cdesc<ConvColKernel<M, E, R, C>>(CK_COL_FILTER, M, E, R, C));               \
  v.push_back(cdesc<ConvColKernel<M, E, R, C>>(CK_COL_SIGNAL, M, E, R, C));               \
  v.push_back(cdesc<ConvColKernel<M, E, R, C, false, true>>(CK_COL_FILTER_H, M, E, R, C)); \
  v.push_back(cdesc<ConvColKernel<M, E, R, C, false, true>>(CK_COL_SIGNAL_H, M, E, R, C));
#define ESTL_XC_ROW(M, E, R, C)                                                \
  v.push_back(cdesc<SpecRowKernel<M, E, R, C>>(CK_SPEC_ROW, M, E, R, C));        \
  v.push_back(cdesc<ConvMidKernel<M, E, R, C>>(CK_MID, M, E, R, C));             \
  v.push_back(cdesc<SpecRowHalfKernel<M, E, R, C>>(CK_SPEC_ROW_H, M, E, R, C));  \
  v.push_back(cdesc<ConvMidHalfKernel<M, E, R, C>>(CK_MID_H, M, E, R, C));
#define ESTL_XC_OUT(M, E, R, C)                                            \
  v.push_back(cdesc<ConvOutKernel<M, E, R, C>>(CK_OUT, M, E, R, C)); \
  v.push_back(cdesc<ConvOutHalfKernel<M, E, R, C>>(CK_OUT_H, M, E, R, C));
#include "conv_list.inc"
    // split-precision (tensor-core) variants of the 16-elements-per-thread tiles
#define ESTL_XC_SINGLE(M, E, R, C)                                                        \
  if constexpr (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog) {                             \
    v.push_back(cdesc<SpecSingleKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(      \
        CK_SPEC_SINGLE, M, E, R, C, 1));                                                                    \
    v.push_back(cdesc<ConvSingleKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(      \
        CK_CONV_SINGLE, M, E, R, C, 1));                                                                    \
    v.push_back(cdesc<SpecPairKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(        \
        CK_SPEC_PAIR, M, E, R, C, 1));                                                                      \
    v.push_back(cdesc<ConvPairKernel<M, E, R, C, (E == 4 && M >= 4 && M <= kConvTcSingleMaxLog)>>(        \
        CK_CONV_PAIR, M, E, R, C, 1));                                                                      \
  }
#define ESTL_XC_COL(M, E, R, C)                                                \
  v.push_back(cdesc<ConvColKernel<M, E, R, C, true>>(CK_COL_FILTER, M, E, R, C, 1)); \
  v.push_back(cdesc<ConvColKernel<M, E, R, C, true>>(CK_COL_SIGNAL, M, E, R, C, 1));
#define ESTL_XC_ROW(M, E, R, C)                                              \
  v.push_back(cdesc<SpecRowKernel<M, E, R, C, true>>(CK_SPEC_ROW, M, E, R, C, 1)); \
  v.push_back(cdesc<ConvMidKernel<M, E, R, C, true>>(CK_MID, M, E, R, C, 1));
#define ESTL_XC_OUT(M, E, R, C) v.push_back(cdesc<ConvOutKernel<M, E, R, C, true>>(CK_OUT, M, E, R, C, 1));
#include "conv_list.inc"
    return v;
  }();
  return t;
}

// every kernel of the table fits the shared memory of one SM
bool conv_table_fits() {
  for (const ConvKernelDesc& d : conv_table())
    if (d.smem_bytes > kMaxConvSmemBytes) return false;
  return true;
}

std::mutex g_conv_attr_mu;

estl_status conv_lookup(const ConvLaunch& l, const ConvKernelDesc** out) {
  static const bool fits = conv_table_fits();
  if (!fits) return fail(ESTL_DEVICE_ERROR, "a convolution kernel needs more shared memory than an SM has");
  for (ConvKernelDesc& d : conv_table()) {
    if (d.kind == l.kind && d.logm == l.logm && d.loge == l.loge && d.logr == l.logr && d.logc == l.logc &&
        d.tc == l.tc) {
      if (!d.attr_set) {
        std::lock_guard<std::mutex> g(g_conv_attr_mu);
        if (!d.attr_set) {
          estl_status s = check_cuda(cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem_bytes),
                                     "cudaFuncSetAttribute(conv)");
          if (s != ESTL_OK) return s;
          d.attr_set = true;
        }
      }
      *out = &d;
      return ESTL_OK;
    }
  }
  return fail(ESTL_UNSUPPORTED_SIZE, "no convolution kernel for launch kind %d logm %d", l.kind, l.logm);
}

}  // namespace

estl_status launch_conv(const ConvLayout& L, const ConvBuffers& b, int which, cudaStream_t stream) {
  Engine& E = engine();
  for (size_t i = 0; i < L.launches.size(); ++i) {
    const ConvLaunch& l = L.launches[i];
    const bool spec_launch = L.is_spectrum_launch[i];
    if (!((spec_launch && (which & 1)) || (!spec_launch && (which & 2)))) continue;
    const ConvKernelDesc* d = nullptr;
    estl_status s = conv_lookup(l, &d);
    if (s != ESTL_OK) return s;
    if (l.grid < 1 || l.grid > INT_MAX) return fail(ESTL_UNSUPPORTED_SIZE, "convolution grid of %lld CTAs", l.grid);
    const long long N = 1LL << l.logn;
    ConvArgs a;
    const bool filt = ck_is_filter(l.kind);
    a.rows = Ptr<const ConvRow>{(filt ? b.filt_rows : b.sig_rows) + l.row_begin, l.row_count};
    a.nrows = l.row_count;
    a.sig = filt ? Ptr<const float>{b.filt, b.filt_elems} : Ptr<const float>{b.sig, b.sig_elems};
    a.spec = Ptr<const cf32>{b.spec, L.spec_elems};
    a.spec_out = Ptr<cf32>{b.spec, L.spec_elems};
    a.out = Ptr<float>{b.out, b.out_elems};
    a.s1 = Ptr<cf32>{b.s1 + l.s_off, l.row_count * N};
    a.s2 = Ptr<cf32>{b.s2 + l.s_off, l.row_count * N};
    a.bank = Ptr<const cf32>{E.bank, kBankSize};
    a.logn = l.logn;
    a.split = l.tc ? L.split : SPLIT_NONE;
    a.shared = L.shared;
    void* args[] = {&a};
    s = launch_pdl(d->fn, l.grid, d->nthreads, args, d->smem_bytes, stream, "cudaLaunchKernelEx(conv)");
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}

ConvBuffers conv_buffers(const ConvLayout& L, void* ws, const float* sig, long long sig_elems, const float* filt,
                         long long filt_elems, float* out) {
  char* w = static_cast<char*>(ws);
  ConvBuffers b;
  b.sig = sig;
  b.sig_elems = sig_elems;
  b.filt = filt;
  b.filt_elems = filt_elems;
  b.out = out;
  b.out_elems = L.out_elems;
  b.filt_rows = reinterpret_cast<const ConvRow*>(w + L.off_filt_rows);
  b.sig_rows = reinterpret_cast<const ConvRow*>(w + L.off_sig_rows);
  b.spec = reinterpret_cast<cf32*>(w + L.off_spec);
  b.s1 = reinterpret_cast<cf32*>(w + L.off_s1);
  b.s2 = reinterpret_cast<cf32*>(w + L.off_s2);
  return b;
}

}  // namespace estl

using namespace estl;

static_assert(sizeof(estl_conv_request) == sizeof(ConvReq), "request layout");

static estl_status conv_layout_from(const estl_conv_request* reqs, int64_t count, int flags, ConvLayout* L,
                                    bool shared) {
  if (count < 1 || count > INT_MAX || !reqs) return fail(ESTL_INVALID_ARG, "need 1..INT_MAX requests");
  if (flags & ~kConvFlagMask) return fail(ESTL_INVALID_ARG, "unknown flags %d", flags);
  std::string err;
  if (!build_conv_layout(reinterpret_cast<const ConvReq*>(reqs), (int)count, flags, L, &err, shared))
    return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  return ESTL_OK;
}

extern "C" {

estl_status estl_conv_workspace_size(const estl_conv_request* reqs, int64_t count, int flags, size_t* bytes) {
  if (!bytes) return fail(ESTL_INVALID_ARG, "NULL output");
  ConvLayout L;
  estl_status s = conv_layout_from(reqs, count, flags, &L, false);
  if (s != ESTL_OK) return s;
  *bytes = L.workspace_bytes;
  return ESTL_OK;
}

estl_status estl_conv_execute(const estl_conv_request* reqs, int64_t count, int flags, const float* d_signals,
                              const float* d_filters, float* d_out, void* d_workspace, size_t workspace_bytes,
                              void* stream) {
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  ConvLayout L;
  s = conv_layout_from(reqs, count, flags, &L, false);
  if (s != ESTL_OK) return s;
  if (!d_signals || !d_filters || !d_out || !d_workspace) return fail(ESTL_INVALID_ARG, "NULL buffer");
  if (workspace_bytes < L.workspace_bytes)
    return fail(ESTL_INVALID_ARG, "workspace of %zu bytes, %zu needed", workspace_bytes, L.workspace_bytes);
  if ((uintptr_t)d_workspace & 255) return fail(ESTL_INVALID_ARG, "workspace must be 256-byte aligned");
  if (((uintptr_t)d_signals | (uintptr_t)d_filters | (uintptr_t)d_out) & 3)
    return fail(ESTL_INVALID_ARG, "signal, filter and output buffers must be 4-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  char* w = static_cast<char*>(d_workspace);
  // descriptors: from pageable host memory, copied before the call returns
  s = check_cuda(cudaMemcpyAsync(w + L.off_filt_rows, L.filt_rows.data(), L.filt_rows.size() * sizeof(ConvRow),
                                 cudaMemcpyHostToDevice, st),
                 "cudaMemcpyAsync(rows)");
  if (s != ESTL_OK) return s;
  s = check_cuda(cudaMemcpyAsync(w + L.off_sig_rows, L.sig_rows.data(), L.sig_rows.size() * sizeof(ConvRow),
                                 cudaMemcpyHostToDevice, st),
                 "cudaMemcpyAsync(rows)");
  if (s != ESTL_OK) return s;
  long long se, fe;
  conv_extents(reinterpret_cast<const ConvReq*>(reqs), (int)count, &se, &fe);
  ConvBuffers b = conv_buffers(L, d_workspace, d_signals, se, d_filters, fe, d_out);
  s = launch_conv(L, b, 3, st);
  if (s != ESTL_OK) return s;
  return check_cuda(cudaStreamSynchronize(st), "convolution");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// conv plan: one filter, `count` signals of one length (Convolution2D_FFT's
// shape, Convolution.h:95-154, in 1D and batched)
// ---------------------------------------------------------------------------
struct estl_conv_plan_s {
  ConvLayout layout;
  std::vector<ConvReq> reqs;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  bool filter_set = false;
  long long signal_len = 0, filter_len = 0, count = 0;
  int flags = 0;
};

extern "C" {

estl_status estl_conv_plan_create(int64_t signal_len, int64_t filter_len, int64_t count, int flags,
                                  estl_conv_plan* plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan pointer");
  *plan = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (signal_len < 1 || filter_len < 1 || count < 1) return fail(ESTL_INVALID_ARG, "lengths and count must be >= 1");
  std::unique_ptr<estl_conv_plan_s> p(new estl_conv_plan_s);
  p->signal_len = signal_len;
  p->filter_len = filter_len;
  p->count = count;
  p->flags = flags;
  const long long out_len = conv_out_len(signal_len, filter_len, flags);
  for (long long i = 0; i < count; ++i) p->reqs.push_back(ConvReq{signal_len, filter_len, i * signal_len, 0, i * out_len});
  s = conv_layout_from(reinterpret_cast<const estl_conv_request*>(p->reqs.data()), count, flags, &p->layout, true);
  if (s != ESTL_OK) return s;
  p->ws_bytes = p->layout.workspace_bytes;
  s = dev_alloc(&p->ws, p->ws_bytes, "convolution plan workspace");
  if (s != ESTL_OK) return s;
  char* w = static_cast<char*>(p->ws);
  s = check_cuda(cudaMemcpy(w + p->layout.off_filt_rows, p->layout.filt_rows.data(),
                            p->layout.filt_rows.size() * sizeof(ConvRow), cudaMemcpyHostToDevice),
                 "cudaMemcpy(rows)");
  if (s == ESTL_OK)
    s = check_cuda(cudaMemcpy(w + p->layout.off_sig_rows, p->layout.sig_rows.data(),
                              p->layout.sig_rows.size() * sizeof(ConvRow), cudaMemcpyHostToDevice),
                   "cudaMemcpy(rows)");
  if (s != ESTL_OK) {
    dev_free(p->ws, p->ws_bytes);
    return s;
  }
  *plan = p.release();
  return ESTL_OK;
}

estl_status estl_conv_plan_set_filter(estl_conv_plan plan, const float* d_filter, void* stream) {
  if (!plan || !d_filter) return fail(ESTL_INVALID_ARG, "NULL plan or filter");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  ConvBuffers b = conv_buffers(plan->layout, plan->ws, nullptr, 0, d_filter, plan->filter_len, nullptr);
  s = launch_conv(plan->layout, b, 1, (cudaStream_t)stream);
  if (s == ESTL_OK) plan->filter_set = true;
  return s;
}

estl_status estl_conv_plan_execute(estl_conv_plan plan, const float* d_signals, float* d_out, void* stream) {
  if (!plan || !d_signals || !d_out) return fail(ESTL_INVALID_ARG, "NULL plan or buffer");
  if (!plan->filter_set) return fail(ESTL_INVALID_ARG, "estl_conv_plan_set_filter has not been called");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  ConvBuffers b = conv_buffers(plan->layout, plan->ws, d_signals, plan->signal_len * plan->count, nullptr, 0, d_out);
  return launch_conv(plan->layout, b, 2, (cudaStream_t)stream);
}

int64_t estl_conv_output_length(int64_t signal_len, int64_t filter_len, int flags) {
  return conv_out_len(signal_len, filter_len, flags);
}

int64_t estl_conv_plan_launches(estl_conv_plan plan) {
  if (!plan) return 0;
  int64_t k = 0;
  for (char c : plan->layout.is_spectrum_launch) k += c ? 0 : 1;
  return k;
}

estl_status estl_conv_plan_destroy(estl_conv_plan plan) {
  if (!plan) return ESTL_OK;
  cudaDeviceSynchronize();
  dev_free(plan->ws, plan->ws_bytes);
  delete plan;
  return ESTL_OK;
}

}  // extern "C"
