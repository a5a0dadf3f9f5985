// noalloc.cu — four-step FFT for callers that cannot allocate device memory.
//
// estl_execute (api.cu) runs transforms longer than 2^14 points as a
// four-step column pass and row pass through plan scratch that estl_init /
// estl_plan_create obtain with cudaMalloc.  Some callers cannot do that:
//  * plugins whose host owns every byte of device memory through its own
//    allocator (a framework's caching allocator, a fixed memory pool), so an
//    extra cudaMalloc either fails or fragments the host's pool;
//  * latency-critical loops, where cudaMalloc / cudaFree may synchronise the
//    device;
//  * hosts that forbid device allocation inside plugin calls altogether.
// estl_execute_noalloc runs four-step column and row kernels with their
// scratch in a fixed file-scope device array and its own twiddle table, so it
// needs neither estl_init nor a plan: the caller passes only the input and
// output buffers.  It runs the plain tiles of the planner's tile shapes, not
// the bulk-load / tensor-copy variants that estl_execute picks for 2^16..2^22:
// the plain tiles have no device-side waits, so a call cannot end with a wait
// that gave up and an error word that nobody reads (this entry point has no
// plan to report one through).
//
// Limits and sharing (also stated in include/estl_cuda.h):
//  * the scratch array holds kNoAllocScratchElems = 2^22 complex64 (32 MiB);
//    every GPU that loads libestl_cuda.so holds it, plus the 4.4 MB twiddle
//    table, until the process exits;
//  * n must be a power of two in [2^14, 2^22]; larger n is rejected;
//  * the set-up of a device (array addresses, twiddle table, kernel
//    attributes) is redone when the device's current context changes, e.g.
//    after cudaDeviceReset;
//  * every call shares the one array and leaves its last contents there.
//    Nothing has to start at zero: the column pass writes every scratch
//    element the row pass then reads.  Calls whose kernels overlap on the
//    GPU (different streams, no ordering between them) race on the array.
#include <cuda.h>

#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.cuh"

namespace estl {

__global__ void bank_init_kernel(cf32* bank);  // api.cu

namespace {

constexpr long long kNoAllocScratchElems = 1LL << 22;
constexpr int kNoAllocMinLog = 14;
constexpr int kNoAllocMaxLog = 22;
constexpr int kMaxDevices = 64;

__device__ __align__(256) cf32 g_noalloc_scratch[kNoAllocScratchElems];
__device__ __align__(256) cf32 g_noalloc_bank[kBankSize];

struct DeviceArrays {
  bool ready = false;
  CUcontext ctx = nullptr;  // the context the set-up below belongs to
  cf32* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  cf32* bank = nullptr;     // device address of g_noalloc_bank on this device
  std::vector<char> attr;   // per column / row kernel: shared-memory attribute set
};

std::mutex g_mu;
DeviceArrays g_dev[kMaxDevices];

// cuCtxGetCurrent from the driver, through the runtime (no -lcuda).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CUcontext current_context() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  CUcontext c = nullptr;
  if (fn) fn(&c);
  return c;
}

// Once per device and context, with that device current: resolve the device
// addresses of the two arrays (in host code their names are host-side
// stand-ins, not device addresses) and fill the twiddle table.  Runs inside
// the first call on the device (and the first call after the context was
// replaced), which therefore must not be inside a stream capture.
estl_status setup_device(int dev, cudaStream_t stream, DeviceArrays** out) {
  std::lock_guard<std::mutex> g(g_mu);
  DeviceArrays& d = g_dev[dev];
  const CUcontext ctx = current_context();
  if (d.ready && d.ctx != ctx) d = DeviceArrays{};  // cudaDeviceReset or a new primary context
  if (!d.ready) {
    void* p = nullptr;
    estl_status s = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    if (s != ESTL_OK) return s;
    d.scratch = static_cast<cf32*>(p);
    s = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_bank), "cudaGetSymbolAddress(twiddle table)");
    if (s != ESTL_OK) return s;
    d.bank = static_cast<cf32*>(p);
    bank_init_kernel<<<(unsigned)((kBankSize + 255) / 256), 256, 0, stream>>>(d.bank);
    s = check_cuda(cudaGetLastError(), "twiddle table launch");
    if (s == ESTL_OK) s = check_cuda(cudaStreamSynchronize(stream), "twiddle table");
    if (s != ESTL_OK) return s;
    const KernelDesc* kd = nullptr;
    d.attr.assign((size_t)(registry_col(&kd) + registry_row(&kd)), 0);
    d.ctx = ctx;
    d.ready = true;
  }
  *out = &d;
  return ESTL_OK;
}

// The plain (no bulk loads, no device waits) column or row kernel of a plan
// step, with its shared-memory attribute set once per device.
estl_status find_desc(const Step& st, DeviceArrays& dev, const KernelDesc** out) {
  const KernelDesc* cols = nullptr;
  const KernelDesc* rows = nullptr;
  const int ncol = registry_col(&cols), nrow = registry_row(&rows);
  const KernelDesc* d = st.kind == STEP_COL ? cols : rows;
  const int n = st.kind == STEP_COL ? ncol : nrow;
  const int base = st.kind == STEP_COL ? 0 : ncol;
  for (int i = 0; i < n; ++i)
    if (d[i].logm == st.logm && d[i].loge == st.loge && d[i].logr == st.logr && d[i].logc == st.logc && !d[i].pipe &&
        !d[i].tc) {
      std::lock_guard<std::mutex> g(g_mu);
      if (!dev.attr[(size_t)(base + i)]) {
        estl_status s = check_cuda(
            cudaFuncSetAttribute(d[i].fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d[i].smem_bytes),
            "cudaFuncSetAttribute");
        if (s != ESTL_OK) return s;
        dev.attr[(size_t)(base + i)] = 1;
      }
      *out = &d[i];
      return ESTL_OK;
    }
  return fail(ESTL_UNSUPPORTED_SIZE, "estl_execute_noalloc: no kernel for a plan step");
}

}  // namespace
}  // namespace estl

using namespace estl;

extern "C" estl_status estl_execute_noalloc(int64_t n, int64_t batch, int direction, const void* d_in, void* d_out,
                                            void* stream) {
  const int logn = ilog2_exact(n);
  if (logn < kNoAllocMinLog || logn > kNoAllocMaxLog)
    return fail(ESTL_UNSUPPORTED_SIZE,
                "estl_execute_noalloc: n = %lld must be a power of two in [2^%d, 2^%d] (its fixed scratch array "
                "holds 2^%d complex elements; use estl_execute for other sizes)",
                (long long)n, kNoAllocMinLog, kNoAllocMaxLog, kNoAllocMaxLog);
  if (batch < 1) return fail(ESTL_INVALID_ARG, "estl_execute_noalloc: batch must be >= 1 (got %lld)", (long long)batch);
  if (direction != ESTL_FORWARD && direction != ESTL_BACKWARD)
    return fail(ESTL_INVALID_ARG, "estl_execute_noalloc: direction must be -1 or +1 (got %d)", direction);
  if (!d_in || !d_out || ((uintptr_t)d_in & 7) || ((uintptr_t)d_out & 7) || d_in == d_out)
    return fail(ESTL_INVALID_ARG, "estl_execute_noalloc: need distinct, 8-byte aligned device buffers");
  int dev = 0;
  estl_status s = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (s != ESTL_OK) return s;
  if (dev < 0 || dev >= kMaxDevices) return fail(ESTL_INVALID_ARG, "device %d out of range", dev);
  cudaStream_t st = (cudaStream_t)stream;
  DeviceArrays* arrays = nullptr;
  s = setup_device(dev, st, &arrays);
  if (s != ESTL_OK) return s;

  PlanChoice choice;
  choice.mode = 2;
  choice.chunk = kNoAllocScratchElems >> logn;  // transforms per column/row pair
  Plan1D plan;
  std::string err;
  if (!make_plan(n, batch, choice, &plan, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  if (plan.scratch_elems > kNoAllocScratchElems)
    return fail(ESTL_UNSUPPORTED_SIZE, "estl_execute_noalloc: plan needs %lld scratch elements (limit %lld)",
                plan.scratch_elems, kNoAllocScratchElems);
  const cf32* in = static_cast<const cf32*>(d_in);
  cf32* out = static_cast<cf32*>(d_out);
  for (const Step& step : plan.steps) {
    if (step.src == BUF_OUT || step.ologr)
      return fail(ESTL_UNSUPPORTED_SIZE, "estl_execute_noalloc: plans of three passes are not supported");
    const KernelDesc* d = nullptr;
    s = find_desc(step, *arrays, &d);
    if (s != ESTL_OK) return s;
    TileArgs a;
    const cf32* src = step.src == BUF_IN ? in : arrays->scratch;
    cf32* dst = step.dst == BUF_OUT ? out : arrays->scratch;
    a.in = Ptr<const cf32>{src + step.src_off, step.src_len};
    a.out = Ptr<cf32>{dst + step.dst_off, step.dst_len};
    a.bank = Ptr<const cf32>{arrays->bank, kBankSize};
    a.rows = step.rows;
    a.logn = step.logn;
    a.logn1 = 0;
    a.sgn = direction == ESTL_FORWARD ? 1.f : -1.f;
    a.grid = step.grid;
    a.split = SPLIT_NONE;
    a.err = nullptr;
    void* args[] = {&a};
    s = check_cuda(cudaLaunchKernel(d->fn, dim3((unsigned)step.grid), dim3(d->nthreads), args, d->smem_bytes, st),
                   "cudaLaunchKernel");
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}
