// stream.cu — the streamed four-step kernels (stream_core.cuh): registry,
// work-list upload and launch.
#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "engine.h"
#include "stream_core.cuh"

namespace estl {

template <class CK, class RK>
__global__ void __launch_bounds__(CK::NT, min_blocks(CK::NT, CK::TL::E)) stream_kernel(StreamArgs a) {
  extern __shared__ float2 estl_stream_smem[];
  __shared__ int slot[2];
  stream_run<CK, RK>(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_stream_smem), slot);
}

namespace {

struct StreamDesc {
  int logn;
  const void* fn;
  int nthreads;
  int smem_bytes;
  int grid;  // resident CTAs on the device (0 = not yet queried)
};

template <class CK, class RK>
StreamDesc sdesc(int logn) {
  const long long smem = CK::SMEM_ELEMS > RK::SMEM_ELEMS ? CK::SMEM_ELEMS : RK::SMEM_ELEMS;
  return StreamDesc{logn, reinterpret_cast<const void*>(&stream_kernel<CK, RK>), CK::NT, (int)(smem * sizeof(cf32)), 0};
}

std::vector<StreamDesc>& stream_table() {
  static std::vector<StreamDesc> t = [] {
    std::vector<StreamDesc> v;
#define ESTL_XS(LOGN, CM, CE, CC, RM, RE, RC) \
  v.push_back(sdesc<ColKernel<CM, CE, 4, CC>, RemapRowKernel<RM, RE, 4, RC>>(LOGN));
#include "stream_list.inc"
    return v;
  }();
  return t;
}

std::mutex g_stream_mu;

estl_status stream_lookup(int logn, StreamDesc** out) {
  for (StreamDesc& d : stream_table()) {
    if (d.logn != logn) continue;
    std::lock_guard<std::mutex> g(g_stream_mu);
    if (!d.grid) {
      estl_status s = check_cuda(cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem_bytes),
                                 "cudaFuncSetAttribute(stream)");
      if (s != ESTL_OK) return s;
      int per_sm = 0;
      s = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, d.fn, d.nthreads, d.smem_bytes),
                     "occupancy(stream)");
      if (s != ESTL_OK) return s;
      d.grid = std::max(1, per_sm) * engine().num_sms;
    }
    *out = &d;
    return ESTL_OK;
  }
  return fail(ESTL_UNSUPPORTED_SIZE, "no streamed four-step kernel for log2 n = %d", logn);
}

}  // namespace

size_t stream_aux_bytes(const Plan1D& plan) {
  if (plan.aux_items == 0) return 0;
  return ((size_t)plan.aux_items * sizeof(PackedItem) + 255) / 256 * 256 + (1 + 2 * (size_t)plan.batch) * 4 + 256;
}

estl_status stream_prepare(const Plan1D& plan, void* aux, size_t aux_bytes, StreamAux* out) {
  out->items = nullptr;
  out->counters = nullptr;
  out->error = nullptr;
  out->nitems = 0;
  out->counter_bytes = 0;
  for (const Step& st : plan.steps) {
    if (st.kind != STEP_STREAM) continue;
    if (aux_bytes < stream_aux_bytes(plan)) return fail(ESTL_DEVICE_ERROR, "stream work list does not fit");
    std::vector<PackedItem> items((size_t)plan.aux_items);
    stream_items(plan.batch, st.logn, st.logm, st.logc, st.rlogc, st.lag, items.data());
    char* w = static_cast<char*>(aux);
    out->items = reinterpret_cast<PackedItem*>(w);
    out->nitems = (long long)items.size();
    out->counters = reinterpret_cast<unsigned int*>(w + (items.size() * sizeof(PackedItem) + 255) / 256 * 256);
    out->counter_bytes = (1 + 2 * (size_t)plan.batch) * 4;
    out->error = reinterpret_cast<int*>(reinterpret_cast<char*>(out->counters) + (out->counter_bytes + 127) / 128 * 128);
    estl_status s = check_cuda(cudaMemcpy(out->items, items.data(), items.size() * sizeof(PackedItem),
                                          cudaMemcpyHostToDevice),
                               "cudaMemcpy(stream work list)");
    if (s != ESTL_OK) return s;
    return check_cuda(cudaMemset(out->error, 0, sizeof(int)), "cudaMemset(stream error flag)");
  }
  return ESTL_OK;
}

estl_status launch_stream(const Step& st, const cf32* in, cf32* out, cf32* scratch, long long scratch_elems,
                          const StreamAux& aux, float sgn, cudaStream_t stream) {
  if (!aux.items) return fail(ESTL_DEVICE_ERROR, "streamed plan without its work list");
  StreamDesc* d = nullptr;
  estl_status s = stream_lookup(st.logn, &d);
  if (s != ESTL_OK) return s;
  s = check_cuda(cudaMemsetAsync(aux.counters, 0, aux.counter_bytes, stream), "cudaMemsetAsync(stream counters)");
  if (s != ESTL_OK) return s;
  const long long n = 1LL << st.logn;
  StreamArgs a;
  a.items = Ptr<const PackedItem>{aux.items, aux.nitems};
  a.nitems = aux.nitems;
  a.in = Ptr<const cf32>{in + st.src_off, st.src_len};
  a.out = Ptr<cf32>{out + st.dst_off, st.dst_len};
  a.scratch = Ptr<cf32>{scratch, scratch_elems};
  a.bank = Ptr<const cf32>{engine().bank, kBankSize};
  a.next = aux.counters;
  a.col_done = aux.counters + 1;
  a.row_done = aux.counters + 1 + st.rows;
  a.error = aux.error;
  a.sgn = sgn;
  a.logn = st.logn;
  a.ring = st.ring;
  a.ncol = (int)(1LL << (st.logn - st.logm - st.logc));
  a.nrow = (int)(1LL << (st.logm - st.rlogc));
  (void)n;
  const long long grid = std::min<long long>(d->grid, aux.nitems);
  void* args[] = {&a};
  return check_cuda(cudaLaunchKernel(d->fn, dim3((unsigned)grid), dim3(d->nthreads), args, d->smem_bytes, stream),
                    "cudaLaunchKernel(stream)");
}

}  // namespace estl
