// api.cu — the C ABI of include/estl_cuda.h: initialisation, plans, device
// and host execution.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "bluestein_core.cuh"
#include "engine.h"
#include "kernels.cuh"
#include "tuner.h"

namespace estl {

// --------------------------------------------------------------------------
// errors
// --------------------------------------------------------------------------
static thread_local std::string t_last_error;

estl_status fail(estl_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return s;
}

estl_status ok() { return ESTL_OK; }

estl_status check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ESTL_OK;
  // The error is reported through the status code; clear the runtime's
  // last-error slot so that the caller's next CUDA call (or another library's)
  // does not trip over an error this call already handled.
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return fail(ESTL_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(ESTL_DEVICE_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

Engine& engine() {
  static Engine e;
  return e;
}

estl_status require_init() {
  Engine& E = engine();
  if (!E.inited) return fail(ESTL_NOT_INITIALIZED, "estl_init has not been called");
  return check_cuda(cudaSetDevice(E.device), "cudaSetDevice");
}

estl_status dev_alloc(void** p, size_t bytes, const char* what) {
  Engine& E = engine();
  *p = nullptr;
  if (bytes == 0) return ESTL_OK;
  size_t prev = E.used.fetch_add(bytes);
  if (prev + bytes > E.budget) {
    E.used.fetch_sub(bytes);
    return fail(ESTL_OUT_OF_MEMORY, "%s: %zu bytes exceed the HBM budget (%zu of %zu bytes in use)", what, bytes,
                prev, E.budget);
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    E.used.fetch_sub(bytes);
    *p = nullptr;
    return check_cuda(e, what);
  }
  return ESTL_OK;
}

void dev_free(void* p, size_t bytes) {
  if (!p) return;
  cudaFree(p);
  engine().used.fetch_sub(bytes);
}

// --------------------------------------------------------------------------
// twiddle bank
// --------------------------------------------------------------------------
// bank[2^k + j] = w_{2^k}^j (k <= kBankLog), then 4096-entry low tables of
// w_N^j for N = 2^(kBankLog+1) .. 2^kMaxLog.  FP64 sincospi, rounded to FP32.
__global__ void bank_init_kernel(cf32* bank) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= kBankSize) return;
  double x;
  if (idx < kBankDirect) {
    if (idx < 2) {
      bank[idx] = cf32{1.f, 0.f};
      return;
    }
    int k = 63 - __clzll(idx);
    long long j = idx - (1LL << k);
    x = -(double)j / (double)(1LL << (k - 1));
  } else {
    long long r = idx - kBankDirect;
    int n = kBankLog + 1 + (int)(r >> kLoLog);
    long long j = r & ((1LL << kLoLog) - 1);
    x = -(double)j / (double)(1LL << (n - 1));
  }
  double s, c;
  sincospi(x, &s, &c);
  bank[idx] = cf32{(float)c, (float)s};
}

// --------------------------------------------------------------------------
// kernel lookup
// --------------------------------------------------------------------------
struct KernelTable {
  std::vector<KernelDesc> descs;
  std::vector<char> attr_set;
  std::vector<int> resident;  // persistent kernels: CTAs resident on the device
};

static KernelTable& ktable() {
  static KernelTable t = [] {
    KernelTable k;
    const KernelDesc* d;
    int n = registry_single(&d);
    k.descs.insert(k.descs.end(), d, d + n);
    n = registry_col(&d);
    k.descs.insert(k.descs.end(), d, d + n);
    n = registry_row(&d);
    k.descs.insert(k.descs.end(), d, d + n);
    k.attr_set.assign(k.descs.size(), 0);
    k.resident.assign(k.descs.size(), 0);
    return k;
  }();
  return t;
}

static std::mutex g_attr_mu;

static estl_status lookup_kernel(const Step& st, int pipe, const KernelDesc** out, int* resident = nullptr) {
  KernelTable& kt = ktable();
  for (size_t i = 0; i < kt.descs.size(); ++i) {
    const KernelDesc& d = kt.descs[i];
    if (d.kind == st.kind && d.logm == st.logm && d.loge == st.loge && d.logr == st.logr && d.logc == st.logc &&
        d.pipe == pipe && d.tc == st.tc && d.cluster == st.cluster && d.csplit == st.csplit) {
      if (!kt.attr_set[i]) {
        std::lock_guard<std::mutex> g(g_attr_mu);
        if (!kt.attr_set[i]) {
          estl_status s = check_cuda(
              cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem_bytes),
              "cudaFuncSetAttribute(max dynamic shared memory)");
          if (s != ESTL_OK) return s;
          if (d.cluster > 3) {  // clusters of more than 8 CTAs are non-portable
            s = check_cuda(cudaFuncSetAttribute(d.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
                           "cudaFuncSetAttribute(non-portable cluster size)");
            if (s != ESTL_OK) return s;
          }
          int per_sm = 0;
          s = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, d.fn, d.nthreads, d.smem_bytes),
                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
          if (s != ESTL_OK) return s;
          kt.resident[i] = std::max(1, per_sm) * engine().num_sms;
          kt.attr_set[i] = 1;
        }
      }
      *out = &d;
      if (resident) *resident = kt.resident[i];
      return ESTL_OK;
    }
  }
  return fail(ESTL_UNSUPPORTED_SIZE, "no kernel instantiated for step kind %d logm %d loge %d logc %d", st.kind,
              st.logm, st.loge, st.logc);
}

estl_status launch_pdl(const void* fn, long long grid, int threads, void** args, int smem, cudaStream_t stream,
                       const char* what, int cluster) {
  // ESTL_NO_PDL=1 launches with plain stream serialisation
  static const bool pdl = [] {
    const char* e = std::getenv("ESTL_NO_PDL");
    return !(e && *e && *e != '0');
  }();
  if (!pdl && !cluster)
    return check_cuda(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3((unsigned)threads), args, (size_t)smem, stream),
                      what);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[2];
  int na = 0;
  if (pdl) {
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  if (cluster) {  // cluster tiles: 2^cluster consecutive CTAs per cluster
    attr[na].id = cudaLaunchAttributeClusterDimension;
    attr[na].val.clusterDim.x = 1u << cluster;
    attr[na].val.clusterDim.y = 1;
    attr[na].val.clusterDim.z = 1;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  return check_cuda(cudaLaunchKernelExC(&cfg, fn, args), what);
}

// cuTensorMapEncodeTiled from the driver, through the runtime (no -lcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// The column pass's view of its input: rows * 2^logm rows of N1 = 2^(logn -
// logm) complex (as 2 N1 floats, pitch N1 * 8 bytes); boxes of C complex x
// min(2^logm, 256) rows.
static estl_status encode_column_map(CUtensorMap* map, const cf32* base, const Step& st) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return fail(ESTL_DEVICE_ERROR, "cuTensorMapEncodeTiled is not available from the driver");
  const long long n1 = 1LL << (st.logn - st.logm);
  const long long height = st.rows << st.logm;
  if (height > (1LL << 31)) return fail(ESTL_UNSUPPORTED_SIZE, "tensor map of %lld rows", height);
  const cuuint64_t dims[2] = {(cuuint64_t)(2 * n1), (cuuint64_t)height};
  const cuuint64_t strides[1] = {(cuuint64_t)(n1 * sizeof(cf32))};
  const cuuint32_t box[2] = {(cuuint32_t)(2 << st.logc), (cuuint32_t)std::min(1 << st.logm, 256)};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<cf32*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ESTL_DEVICE_ERROR, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ESTL_OK;
}

estl_status prepare_steps(const Plan1D& plan) {
  for (const Step& st : plan.steps) {
    if (st.kind == STEP_COPY) continue;
    const KernelDesc* d = nullptr;
    estl_status s = lookup_kernel(st, st.pipe, &d);
    if (s != ESTL_OK) return s;
    if (st.pipe) {
      s = lookup_kernel(st, 0, &d);  // the plain tile, run when buffers are not 16-byte aligned
      if (s != ESTL_OK) return s;
    }
  }
  return ESTL_OK;
}

estl_status take_bulk_wait_error() {
  long long e = 0;
  estl_status s = check_cuda(cudaMemcpy(&e, engine().dev_err, sizeof(e), cudaMemcpyDeviceToHost), "cudaMemcpy(error word)");
  if (s != ESTL_OK || !e) return s;
  cudaMemset(engine().dev_err, 0, sizeof(long long));
  if (e & kErrCopiesInFlight)
    return fail(ESTL_DEVICE_ERROR, "a bulk-load wait gave up (tile %lld) and its copies in flight did not drain",
                (e & ~kErrCopiesInFlight) - 1);
  return fail(ESTL_TIMEOUT, "a bulk-load wait gave up (tile %lld)", e - 1);
}

estl_status launch_steps(const Plan1D& plan, const cf32* in, cf32* out, cf32* scratch, float sgn,
                         cudaStream_t stream, const long long* xoff, long long extent) {
  Engine& E = engine();
  for (const Step& st : plan.steps) {
    const cf32* src = st.src == BUF_IN ? in : (st.src == BUF_SCRATCH ? scratch : out);
    cf32* dst = st.dst == BUF_OUT ? out : scratch;
    if (st.kind == STEP_COPY) {
      estl_status s = check_cuda(cudaMemcpyAsync(dst + st.dst_off, src + st.src_off, st.rows * sizeof(cf32),
                                                 cudaMemcpyDeviceToDevice, stream),
                                 "cudaMemcpyAsync(copy step)");
      if (s != ESTL_OK) return s;
      continue;
    }
    // persistent kernels move 16-byte bulk copies: they need 16-byte aligned data
    const bool aligned = !(((uintptr_t)(src + st.src_off) | (uintptr_t)(dst + st.dst_off)) & 15);
    const int pipe = aligned ? st.pipe : 0;
    const KernelDesc* d = nullptr;
    int resident = 0;
    estl_status s = lookup_kernel(st, pipe, &d, &resident);
    if (s != ESTL_OK) return s;
    if (st.grid < 1 || st.grid > INT_MAX) return fail(ESTL_UNSUPPORTED_SIZE, "grid of %lld CTAs", st.grid);
    const long long grid = pipe ? std::min<long long>(st.grid, resident) : st.grid;
    TileArgs a;
    a.in = Ptr<const cf32>{src + st.src_off, st.src_len};
    a.out = Ptr<cf32>{dst + st.dst_off, st.dst_len};
    a.bank = Ptr<const cf32>{E.bank, kBankSize};
    a.rows = st.rows;
    a.logn = st.logn;
    a.logn1 = 0;
    a.sgn = sgn;
    a.grid = grid;
    a.split = st.tc ? plan.choice.split : SPLIT_NONE;
    a.err = E.dev_err;
    a.ologr = st.ologr;
    if (st.ologr) a.sgn = 1.f;  // middle pass of three: its input is conjugated already
    if (xoff) {
      // transforms at the caller's offsets: whole buffers, the step's transforms' offsets
      if (d->tmap || st.src == BUF_OUT || st.ologr)
        return fail(ESTL_UNSUPPORTED_SIZE, "a plan step that cannot read transforms through offsets");
      const long long n = 1LL << st.logn;
      const long long first = st.src == BUF_IN ? st.src_off / n : st.dst_off / n;
      if (st.src == BUF_IN) a.in = Ptr<const cf32>{in, extent};
      if (st.dst == BUF_OUT) a.out = Ptr<cf32>{out, extent};
      a.xoff = Ptr<const long long>{xoff + first, st.rows};
    }
    alignas(64) CUtensorMap map;
    if (d->tmap) {
      s = encode_column_map(&map, src + st.src_off, st);
      if (s != ESTL_OK) return s;
    }
    void* args[] = {&a, &map};
    // persistent bulk-load kernels keep plain stream order (measured: with
    // programmatic launch their three-pass chains ran 1-4% slower)
    s = pipe ? check_cuda(cudaLaunchKernel(d->fn, dim3((unsigned)grid), dim3(d->nthreads), args, d->smem_bytes, stream),
                          "cudaLaunchKernel")
             : launch_pdl(d->fn, grid, d->nthreads, args, d->smem_bytes, stream, "cudaLaunchKernelEx", d->cluster);
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}

}  // namespace estl

using namespace estl;

// --------------------------------------------------------------------------
// plans
// --------------------------------------------------------------------------
struct estl_plan_s {
  Plan1D layout;
  float sgn = 1.f;
  int direction = ESTL_FORWARD;
  cf32* scratch = nullptr;
  size_t scratch_bytes = 0;
  std::mutex mu;
  std::mutex host_mu;  // one host pipeline run at a time (staging buffers, chunk plans)
  cudaEvent_t done = nullptr;  // last execute of this plan (scratch reuse order)
  bool done_recorded = false;
  // host pipeline (lazily created by estl_execute_host)
  bool host_ready = false;
  long long host_chunk = 0;
  Plan1D host_plan_full, host_plan_tail;
  cf32* din[2] = {nullptr, nullptr};
  cf32* dout[2] = {nullptr, nullptr};
  size_t stage_bytes = 0;
  cudaStream_t st[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_h2d[2] = {}, ev_comp[2] = {}, ev_d2h[2] = {};
  // the smaller chunks that open and close a host pipeline (estl_execute_host):
  // chunk transforms -> plan (and its streamed work list)
  struct RampChunk {
    Plan1D lay;
  };
  std::unordered_map<long long, RampChunk> ramp;
  // other host layouts (estl_execute_layout / estl_execute_host_layout):
  // interleaved staging of the device path, raw-layout staging of the host path
  cf32* lay_in = nullptr;
  cf32* lay_out = nullptr;
  size_t lay_bytes = 0;
  float* hlay_in[2] = {nullptr, nullptr};
  float* hlay_out[2] = {nullptr, nullptr};
  size_t hlay_bytes = 0;
  // Bluestein plans: chirp (N), scaled kernel spectrum (M), two work buffers
  cf32* blue_chirp = nullptr;
  cf32* blue_spec = nullptr;
  cf32* blue_a = nullptr;
  cf32* blue_c = nullptr;
  size_t blue_chirp_bytes = 0, blue_spec_bytes = 0, blue_work_bytes = 0;
  // a bounded wait gave up with bulk copies possibly still in flight
  // (estl_plan_check): later executes are refused
  bool unusable = false;
  // per-launch profiling (estl_plan_set_profiling)
  bool profiling = false;
  struct Rec {
    int kind;
    double bytes;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> event_pool;
  long long prof_launches[kStepKinds] = {};
  double prof_ms[kStepKinds] = {}, prof_bytes[kStepKinds] = {};
};

static std::mutex g_plans_mu;
static std::unordered_set<estl_plan> g_plans;

static void plan_release(estl_plan p) {
  if (!p) return;
  dev_free(p->scratch, p->scratch_bytes);
  dev_free(p->blue_chirp, p->blue_chirp_bytes);
  dev_free(p->blue_spec, p->blue_spec_bytes);
  dev_free(p->blue_a, p->blue_work_bytes);
  dev_free(p->blue_c, p->blue_work_bytes);
  dev_free(p->lay_in, p->lay_bytes);
  dev_free(p->lay_out, p->lay_bytes);
  for (int s = 0; s < 2; ++s) {
    dev_free(p->hlay_in[s], p->hlay_bytes);
    dev_free(p->hlay_out[s], p->hlay_bytes);
  }
  for (int s = 0; s < 2; ++s) {
    dev_free(p->din[s], p->stage_bytes);
    dev_free(p->dout[s], p->stage_bytes);
    if (p->ev_h2d[s]) cudaEventDestroy(p->ev_h2d[s]);
    if (p->ev_comp[s]) cudaEventDestroy(p->ev_comp[s]);
    if (p->ev_d2h[s]) cudaEventDestroy(p->ev_d2h[s]);
  }
  for (int s = 0; s < 3; ++s)
    if (p->st[s]) cudaStreamDestroy(p->st[s]);
  if (p->done) cudaEventDestroy(p->done);
  for (auto& r : p->pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : p->event_pool) cudaEventDestroy(e);
  delete p;
}

extern "C" {

estl_status estl_init(int device, size_t hbm_budget_bytes) {
  Engine& E = engine();
  std::lock_guard<std::mutex> g(E.mu);
  if (E.inited) {
    if (device != E.device) return fail(ESTL_INVALID_ARG, "already initialised on device %d", E.device);
    if (hbm_budget_bytes) E.budget = hbm_budget_bytes;
    return ESTL_OK;
  }
  int count = 0;
  estl_status s = check_cuda(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (s != ESTL_OK) return s;
  if (device < 0 || device >= count) return fail(ESTL_INVALID_ARG, "device %d not present (%d devices)", device, count);
  s = check_cuda(cudaSetDevice(device), "cudaSetDevice");
  if (s != ESTL_OK) return s;
  size_t free_b = 0, total_b = 0;
  s = check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  if (s != ESTL_OK) return s;
  cudaDeviceProp prop;
  s = check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (s != ESTL_OK) return s;
  if (prop.major < 10) return fail(ESTL_DEVICE_ERROR, "device %d is sm_%d%d; the library is compiled for sm_103a", device, prop.major, prop.minor);
  E.device = device;
  E.num_sms = prop.multiProcessorCount;
  E.budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)(0.9 * (double)free_b);
  E.used = 0;
  void* b = nullptr;
  E.inited = true;  // dev_alloc needs the budget
  s = dev_alloc(&b, kBankSize * sizeof(cf32), "twiddle bank");
  if (s != ESTL_OK) {
    E.inited = false;
    return s;
  }
  E.bank = (cf32*)b;
  {
    void* w = nullptr;
    s = dev_alloc(&w, 256, "error word");
    if (s != ESTL_OK) return s;
    E.dev_err = (long long*)w;
    s = check_cuda(cudaMemset(E.dev_err, 0, sizeof(long long)), "cudaMemset(error word)");
    if (s != ESTL_OK) return s;
  }
  bank_init_kernel<<<(unsigned)((kBankSize + 255) / 256), 256>>>(E.bank);
  s = check_cuda(cudaGetLastError(), "bank_init_kernel launch");
  if (s == ESTL_OK) s = check_cuda(cudaDeviceSynchronize(), "bank_init_kernel");
  if (s != ESTL_OK) {
    dev_free(E.bank, kBankSize * sizeof(cf32));
    E.bank = nullptr;
    E.inited = false;
    return s;
  }
  tuner_load_cache();
  return ESTL_OK;
}

estl_status estl_shutdown(void) {
  Engine& E = engine();
  {
    std::lock_guard<std::mutex> g(g_plans_mu);
    for (estl_plan p : g_plans) plan_release(p);
    g_plans.clear();
  }
  std::lock_guard<std::mutex> g(E.mu);
  if (!E.inited) return ESTL_OK;
  cudaDeviceSynchronize();
  dev_free(E.bank, kBankSize * sizeof(cf32));
  E.bank = nullptr;
  dev_free(E.dev_err, 256);
  E.dev_err = nullptr;
  E.inited = false;
  return ESTL_OK;
}

const char* estl_last_error(void) { return t_last_error.c_str(); }

const char* estl_status_string(estl_status s) {
  switch (s) {
    case ESTL_OK: return "ESTL_OK";
    case ESTL_INVALID_ARG: return "ESTL_INVALID_ARG";
    case ESTL_UNSUPPORTED_SIZE: return "ESTL_UNSUPPORTED_SIZE";
    case ESTL_OUT_OF_MEMORY: return "ESTL_OUT_OF_MEMORY";
    case ESTL_ADMISSION_REJECTED: return "ESTL_ADMISSION_REJECTED";
    case ESTL_DEVICE_ERROR: return "ESTL_DEVICE_ERROR";
    case ESTL_TIMEOUT: return "ESTL_TIMEOUT";
    case ESTL_NOT_INITIALIZED: return "ESTL_NOT_INITIALIZED";
  }
  return "ESTL_UNKNOWN";
}

int64_t estl_max_batch(int64_t n) {
  Engine& E = engine();
  if (!E.inited || n < 1) return 0;
  size_t fixed = 0;
  if (ilog2_exact(n) < 0) {
    // Bluestein: chirp (n), kernel spectrum (M), two work buffers and the
    // inner plan's scratch of at most 2^26 elements each, held once per plan
    if (n < 3 || n > (1LL << (kBluesteinMaxLogM - 1))) return 0;
    fixed = sizeof(cf32) * ((size_t)n + (size_t)bluestein_m(n) + 3 * ((size_t)1 << 26));
  } else if (ilog2_exact(n) > kMaxLogN) {
    return 0;
  }
  const size_t used = E.used.load() + fixed;
  if (used >= E.budget) return 0;
  long long b = (long long)((E.budget - used) / (3 * sizeof(cf32) * (size_t)n));
  return b > INT32_MAX ? INT32_MAX : b;
}

static estl_status plan_create_impl(int64_t n, int64_t batch, int direction, int precision,
                                    const estl_plan_options* opt, estl_plan* plan);

estl_status estl_plan_create(int64_t n, int64_t batch, int direction, int precision, estl_plan* plan) {
  return plan_create_impl(n, batch, direction, precision, nullptr, plan);
}

estl_status estl_plan_create_ex(int64_t n, int64_t batch, int direction, int precision,
                                const estl_plan_options* options, estl_plan* plan) {
  if (options && (options->mode < 0 || options->mode > 4 || options->mode == 3 || options->lag != 0 ||
                  options->chunk < 0))
    return fail(ESTL_INVALID_ARG, "bad plan options (mode %d, lag %d, chunk %lld)", options->mode, options->lag,
                (long long)options->chunk);
  return plan_create_impl(n, batch, direction, precision, options, plan);
}

static estl_status plan_finish(std::unique_ptr<estl_plan_s> p, int direction, estl_plan* plan);

// ---- Bluestein plans (bluestein_core.cuh) ---------------------------------
static int flat_grid(long long total) {
  const long long blocks = (total + 255) / 256;
  return (int)std::max(1LL, std::min<long long>(blocks, 152LL * 16));
}

__global__ void blue_chirp_kernel(cf32* chirp, long long N) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    chirp[i] = bluestein_chirp(i, N);
}

__global__ void blue_kernel_kernel(const cf32* chirp, cf32* b, long long N, long long M) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    b[i] = bluestein_kernel_elem(chirp, i, N, M);
}

__global__ void blue_scale_kernel(cf32* v, long long M, float s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    v[i] = cf32{v[i].x * s, v[i].y * s};
}

// a[b][m] for `count` transforms of length N into rows of length M
__global__ void blue_pre_kernel(const cf32* __restrict__ x, cf32* __restrict__ a, const cf32* __restrict__ chirp,
                                long long N, int logm, long long count, float sgn) {
  const long long total = count << logm, mask = (1LL << logm) - 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    a[i] = bluestein_pre(x + (i >> logm) * N, chirp, i & mask, N, sgn);
}

__global__ void blue_mul_kernel(cf32* c, const cf32* __restrict__ spec, int logm, long long count) {
  const long long total = count << logm, mask = (1LL << logm) - 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    c[i] = cmul(c[i], spec[i & mask]);
}

__global__ void blue_post_kernel(const cf32* __restrict__ c, cf32* __restrict__ y, const cf32* __restrict__ chirp,
                                 long long N, int logm, long long count, float sgn) {
  const long long total = count * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / N, k = i - b * N;
    y[i] = bluestein_post(c + (b << logm), chirp, k, sgn);
  }
}

}  // extern "C"

// Bluestein tile kernels (bluestein_core.cuh): the fused one-pass kernel of
// M <= 2^14 (one tile shape per M, ESTL_BLUE_TILES) and the three four-step
// kernels of M <= 2^22 (the convolution's tile shapes, conv_list.inc).
template <class K>
__global__ void __launch_bounds__(K::NT, K::MIN_BLOCKS) bluestein_tile_kernel(BlueArgs a) {
  extern __shared__ float2 estl_blue_smem[];
  K::run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_blue_smem));
}

namespace {
// kind 0: fused one-pass kernel (logm = log2 M); 1 / 2 / 3: four-step column,
// middle and output kernels (logm = their tile length)
struct BlueDesc {
  int kind, logm, logc, nt, smem_bytes;
  const void* fn;
  bool attr_set;
};
std::mutex g_blue_mu;
template <class K>
BlueDesc blue_desc(int kind, int m, int c) {
  return BlueDesc{kind, m, c, K::NT, (int)(K::SMEM_ELEMS * sizeof(cf32)),
                  reinterpret_cast<const void*>(&bluestein_tile_kernel<K>), false};
}
std::vector<BlueDesc>& blue_table() {
  static std::vector<BlueDesc> t = [] {
    std::vector<BlueDesc> v;
#define ESTL_BLUE_DESC(M, E, R, C) v.push_back(blue_desc<BlueSingleKernel<M, E, R, C>>(0, M, C));
    ESTL_BLUE_TILES(ESTL_BLUE_DESC)
#undef ESTL_BLUE_DESC
#define ESTL_XC_COL(M, E, R, C) v.push_back(blue_desc<BlueColKernel<M, E, R, C>>(1, M, C));
#define ESTL_XC_ROW(M, E, R, C) v.push_back(blue_desc<BlueMidKernel<M, E, R, C>>(2, M, C));
#define ESTL_XC_OUT(M, E, R, C) v.push_back(blue_desc<BlueOutKernel<M, E, R, C>>(3, M, C));
#include "conv_list.inc"
    return v;
  }();
  return t;
}

estl_status blue_launch(int kind, int logm, long long units, const BlueArgs& a, cudaStream_t st) {
  BlueDesc* d = nullptr;
  for (BlueDesc& b : blue_table())
    if (b.kind == kind && b.logm == logm) d = &b;
  if (!d) return fail(ESTL_UNSUPPORTED_SIZE, "no Bluestein kernel of kind %d for a tile of 2^%d", kind, logm);
  if (!d->attr_set) {
    std::lock_guard<std::mutex> g(g_blue_mu);
    if (!d->attr_set) {
      estl_status s = check_cuda(cudaFuncSetAttribute(d->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, d->smem_bytes),
                                 "cudaFuncSetAttribute(Bluestein)");
      if (s != ESTL_OK) return s;
      d->attr_set = true;
    }
  }
  // units: transforms (fused kernel) or tiles of C columns / rows (four-step)
  const long long grid = kind == 0 ? (units + (1LL << d->logc) - 1) >> d->logc : units >> d->logc;
  if (grid < 1 || grid > INT_MAX) return fail(ESTL_UNSUPPORTED_SIZE, "Bluestein grid of %lld CTAs", grid);
  BlueArgs args = a;
  void* kargs[] = {&args};
  return check_cuda(cudaLaunchKernel(d->fn, dim3((unsigned)grid), dim3((unsigned)d->nt), kargs, (size_t)d->smem_bytes,
                                     st),
                    "Bluestein kernel");
}
}  // namespace

static BlueArgs blue_args(estl_plan p, long long count, const cf32* in, cf32* out) {
  const long long N = p->layout.n, M = p->layout.blue_m;
  BlueArgs a;
  a.in = Ptr<const cf32>{in, count * N};
  a.out = Ptr<cf32>{out, count * N};
  a.chirp = Ptr<const cf32>{p->blue_chirp, N};
  a.spec = Ptr<const cf32>{p->blue_spec, M};
  a.bank = Ptr<const cf32>{engine().bank, kBankSize};
  a.n = N;
  a.count = count;
  a.sgn = p->sgn;
  a.logm = ilog2_exact(M);
  return a;
}

// `count` transforms through the fused kernel of M.
static estl_status run_bluestein_fused(estl_plan p, long long count, const cf32* in, cf32* out, cudaStream_t st) {
  const BlueArgs a = blue_args(p, count, in, out);
  return blue_launch(0, a.logm, count, a, st);
}

// Four-step: chunks of blue_chunk transforms, the scratch in the work buffers.
static estl_status run_bluestein_four_step(estl_plan p, long long count, const cf32* in, cf32* out,
                                           cudaStream_t st) {
  const long long N = p->layout.n, M = p->layout.blue_m, cmax = p->layout.blue_chunk;
  const int logm = ilog2_exact(M), logn2 = bluestein_logn2(logm), logn1 = logm - logn2;
  for (long long b0 = 0; b0 < count; b0 += cmax) {
    const long long c = std::min(cmax, count - b0);
    BlueArgs a = blue_args(p, c, in + b0 * N, out + b0 * N);
    a.s1 = Ptr<cf32>{p->blue_a, c * M};
    a.s2 = Ptr<cf32>{p->blue_c, c * M};
    estl_status s = blue_launch(1, logn2, c << logn1, a, st);  // C columns of N2 per CTA
    if (s == ESTL_OK) s = blue_launch(2, logn1, c << logn2, a, st);  // C rows of N1 per CTA
    if (s == ESTL_OK) s = blue_launch(3, logn2, c << logn1, a, st);  // C rows of N2 per CTA
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}

// Bp[k2*N1 + k1] = Bs[k2 + N2*k1]: the kernel spectrum in the order the
// four-step middle kernel reads it.
__global__ void blue_permute_kernel(const cf32* __restrict__ bs, cf32* __restrict__ bp, int logn1, int logn2) {
  const long long m = 1LL << (logn1 + logn2);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const long long k2 = i >> logn1, k1 = i & ((1LL << logn1) - 1);
    bp[i] = bs[k2 + (k1 << logn2)];
  }
}

extern "C" {

// Chirp, the kernel spectrum FFT_M(b) / M and the work buffers of a plan
// (one M-element buffer for the fused kernel's set-up).
static estl_status bluestein_setup(estl_plan_s* p) {
  const long long N = p->layout.n, M = p->layout.blue_m;
  const long long cmax = bluestein_fused(M) ? 1 : p->layout.blue_chunk;
  p->blue_chirp_bytes = (size_t)N * sizeof(cf32);
  p->blue_spec_bytes = (size_t)M * sizeof(cf32);
  p->blue_work_bytes = (size_t)(cmax * M) * sizeof(cf32);
  estl_status s = dev_alloc((void**)&p->blue_chirp, p->blue_chirp_bytes, "Bluestein chirp");
  if (s == ESTL_OK) s = dev_alloc((void**)&p->blue_spec, p->blue_spec_bytes, "Bluestein spectrum");
  if (s == ESTL_OK) s = dev_alloc((void**)&p->blue_a, p->blue_work_bytes, "Bluestein work");
  if (s == ESTL_OK) s = dev_alloc((void**)&p->blue_c, p->blue_work_bytes, "Bluestein work");
  if (s != ESTL_OK) return s;
  Plan1D one;
  std::string err;
  if (!make_plan(M, 1, PlanChoice{}, &one, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  if ((size_t)one.scratch_elems * sizeof(cf32) > p->scratch_bytes)
    return fail(ESTL_DEVICE_ERROR, "Bluestein set-up needs more scratch than the plan holds");
  cudaStream_t st = 0;  // legacy default stream: ordered with every blocking stream
  blue_chirp_kernel<<<flat_grid(N), 256, 0, st>>>(p->blue_chirp, N);
  blue_kernel_kernel<<<flat_grid(M), 256, 0, st>>>(p->blue_chirp, p->blue_a, N, M);
  s = check_cuda(cudaGetLastError(), "Bluestein set-up");
  if (s == ESTL_OK) s = launch_steps(one, p->blue_a, p->blue_spec, p->scratch, 1.f, st);
  if (s != ESTL_OK) return s;
  blue_scale_kernel<<<flat_grid(M), 256, 0, st>>>(p->blue_spec, M, 1.f / (float)M);
  s = check_cuda(cudaGetLastError(), "Bluestein set-up");
  if (s == ESTL_OK && bluestein_four_step(M)) {
    // the four-step middle kernel reads the spectrum permuted (the work
    // buffer is free until the first execute)
    const int logm = ilog2_exact(M), logn2 = bluestein_logn2(logm);
    s = check_cuda(cudaMemcpyAsync(p->blue_a, p->blue_spec, (size_t)M * sizeof(cf32), cudaMemcpyDeviceToDevice, st),
                   "Bluestein set-up");
    if (s == ESTL_OK) {
      blue_permute_kernel<<<flat_grid(M), 256, 0, st>>>(p->blue_a, p->blue_spec, logm - logn2, logn2);
      s = check_cuda(cudaGetLastError(), "Bluestein set-up");
    }
  }
  if (s == ESTL_OK) s = check_cuda(cudaStreamSynchronize(st), "Bluestein set-up");
  return s;
}

// `count` transforms of a Bluestein plan: pre-multiply, M-point FFT, spectrum
// multiply, M-point inverse FFT, post-multiply, in chunks of blue_chunk.
static estl_status run_bluestein(estl_plan p, long long count, const cf32* in, cf32* out, cudaStream_t st) {
  if (bluestein_fused(p->layout.blue_m)) return run_bluestein_fused(p, count, in, out, st);
  if (bluestein_four_step(p->layout.blue_m)) return run_bluestein_four_step(p, count, in, out, st);
  const long long N = p->layout.n, M = p->layout.blue_m, cmax = p->layout.blue_chunk;
  const int logm = ilog2_exact(M);
  for (long long b0 = 0; b0 < count; b0 += cmax) {
    const long long c = std::min(cmax, count - b0);
    Plan1D inner;
    std::string err;
    if (!make_plan(M, c, PlanChoice{}, &inner, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
    blue_pre_kernel<<<flat_grid(c * M), 256, 0, st>>>(in + b0 * N, p->blue_a, p->blue_chirp, N, logm, c, p->sgn);
    estl_status s = check_cuda(cudaGetLastError(), "Bluestein pre-multiply");
    if (s == ESTL_OK) s = launch_steps(inner, p->blue_a, p->blue_c, p->scratch, 1.f, st);
    if (s != ESTL_OK) return s;
    blue_mul_kernel<<<flat_grid(c * M), 256, 0, st>>>(p->blue_c, p->blue_spec, logm, c);
    s = check_cuda(cudaGetLastError(), "Bluestein spectrum multiply");
    if (s == ESTL_OK) s = launch_steps(inner, p->blue_c, p->blue_a, p->scratch, -1.f, st);
    if (s != ESTL_OK) return s;
    blue_post_kernel<<<flat_grid(c * N), 256, 0, st>>>(p->blue_a, out + b0 * N, p->blue_chirp, N, logm, c, p->sgn);
    s = check_cuda(cudaGetLastError(), "Bluestein post-multiply");
    if (s != ESTL_OK) return s;
  }
  return ESTL_OK;
}

static estl_status plan_create_impl(int64_t n, int64_t batch, int direction, int precision,
                                    const estl_plan_options* opt, estl_plan* plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "plan output pointer is NULL");
  *plan = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (direction != ESTL_FORWARD && direction != ESTL_BACKWARD)
    return fail(ESTL_INVALID_ARG, "direction must be ESTL_FORWARD (-1) or ESTL_BACKWARD (+1), got %d", direction);
  if (precision < ESTL_PREC_FP32 || precision > ESTL_PREC_SPLIT_BF16X3)
    return fail(ESTL_INVALID_ARG, "unknown precision %d", precision);
  if (batch < 1) return fail(ESTL_INVALID_ARG, "batch must be >= 1 (got %lld)", (long long)batch);
  int logn = ilog2_exact(n);
  if (logn < 0 && n > 2) {
    // any other length: Bluestein over power-of-two FFTs (FP32, planner defaults)
    if (precision != ESTL_PREC_FP32)
      return fail(ESTL_INVALID_ARG, "lengths that are not powers of two run in FP32 (precision %d)", precision);
    if (opt && opt->mode != 0) return fail(ESTL_INVALID_ARG, "plan options apply to power-of-two lengths");
    std::unique_ptr<estl_plan_s> p(new estl_plan_s);
    std::string err;
    if (!make_plan_bluestein(n, batch, &p->layout, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
    return plan_finish(std::move(p), direction, plan);
  }
  if (logn < 0 || logn > kMaxLogN)
    return fail(ESTL_UNSUPPORTED_SIZE, "transform length %lld must be at least 1 and at most 2^%d", (long long)n,
                kMaxLogN);
  PlanChoice choice;
  if (opt && opt->mode != 0) {
    choice.mode = opt->mode;
    choice.chunk = opt->chunk;
    if (opt->explicit_tiles) {
      choice.logn2 = opt->split_log2;
      choice.single_loge = opt->single_loge;
      choice.single_logc = opt->single_logc;
      choice.col_loge = opt->col_loge;
      choice.col_logc = opt->col_logc;
      choice.row_loge = opt->row_loge;
      choice.row_logc = opt->row_logc;
      choice.pipe = opt->pipelined < 0 ? 0 : opt->pipelined;
      choice.logn3 = opt->split2_log2;
      choice.single_logr = opt->single_logr;
      choice.col_logr = opt->col_logr;
      choice.row_logr = opt->row_logr;
      choice.single_cluster = opt->single_cluster_log2;
    }
  } else {
    if (precision == ESTL_PREC_FP32) tuner_lookup(n, batch, &choice);
  }
  choice.split = precision;  // ESTL_PREC_SPLIT_* == SplitKind
  std::unique_ptr<estl_plan_s> p(new estl_plan_s);
  std::string err;
  if (opt && opt->mode != 0) {
    if (!make_plan(n, batch, choice, &p->layout, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  } else if (!make_plan(n, batch, choice, &p->layout, &err)) {
    // a stale tuning entry must not make a valid size fail: fall back to defaults
    PlanChoice dflt;
    dflt.split = precision;
    if (!make_plan(n, batch, dflt, &p->layout, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  }
  return plan_finish(std::move(p), direction, plan);
}

// Device buffers, work list and ordering event of a plan whose layout is set.
static estl_status plan_finish(std::unique_ptr<estl_plan_s> p, int direction, estl_plan* plan) {
  estl_status s;
  p->direction = direction;
  p->sgn = direction == ESTL_FORWARD ? 1.f : -1.f;
  p->scratch_bytes = (size_t)p->layout.scratch_elems * sizeof(cf32);
  s = dev_alloc((void**)&p->scratch, p->scratch_bytes, "plan scratch");
  if (s != ESTL_OK) return s;
  if (p->layout.blue_m > 0) {
    s = bluestein_setup(p.get());
    if (s != ESTL_OK) {
      plan_release(p.release());
      return s;
    }
  }
  s = check_cuda(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming), "cudaEventCreate");
  if (s != ESTL_OK) {
    plan_release(p.release());
    return s;
  }
  estl_plan out = p.release();
  {
    std::lock_guard<std::mutex> g(g_plans_mu);
    g_plans.insert(out);
  }
  *plan = out;
  return ESTL_OK;
}

estl_status estl_plan2d_create(int64_t xdim, int64_t ydim, int64_t batch, int direction, int precision,
                               estl_plan* plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "plan output pointer is NULL");
  *plan = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (direction != ESTL_FORWARD && direction != ESTL_BACKWARD)
    return fail(ESTL_INVALID_ARG, "direction must be ESTL_FORWARD (-1) or ESTL_BACKWARD (+1), got %d", direction);
  if (precision != ESTL_PREC_FP32) return fail(ESTL_INVALID_ARG, "2D transforms run in FP32 (precision %d)", precision);
  PlanChoice choice;
  if (xdim > 0 && batch > 0 && ydim > 0 && batch <= (1LL << kMaxTotalLog) / ydim)
    tuner_lookup(xdim, ydim * batch, &choice);  // the row FFTs' tuned plan
  std::unique_ptr<estl_plan_s> p(new estl_plan_s);
  std::string err;
  if (!make_plan2d(xdim, ydim, batch, choice, &p->layout, &err) &&
      !make_plan2d(xdim, ydim, batch, PlanChoice{}, &p->layout, &err))
    return fail(xdim < 1 || ydim < 1 || batch < 1 ? ESTL_INVALID_ARG : ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  return plan_finish(std::move(p), direction, plan);
}

estl_status estl_plan_destroy(estl_plan plan) {
  if (!plan) return ESTL_OK;
  {
    std::lock_guard<std::mutex> g(g_plans_mu);
    if (!g_plans.erase(plan)) return fail(ESTL_INVALID_ARG, "unknown plan handle");
  }
  // wait for the plan's last execute (an event last recorded inside a stream
  // capture has nothing to wait for here and only reports an error, which is
  // cleared)
  if (plan->done_recorded && cudaEventSynchronize(plan->done) != cudaSuccess) cudaGetLastError();
  plan_release(plan);
  return ESTL_OK;
}

estl_status estl_plan_describe(estl_plan plan, char* buf, size_t len) {
  if (!plan || !buf || len == 0) return fail(ESTL_INVALID_ARG, "NULL plan or buffer");
  std::string d = plan->layout.describe();
  std::snprintf(buf, len, "%s", d.c_str());
  return ESTL_OK;
}

estl_status estl_plan_check(estl_plan plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  estl_status s = check_cuda(cudaDeviceSynchronize(), "plan execute");
  if (s != ESTL_OK) return s;
  long long e = 0;
  s = check_cuda(cudaMemcpy(&e, engine().dev_err, sizeof(e), cudaMemcpyDeviceToHost), "cudaMemcpy(error word)");
  if (s != ESTL_OK) return s;
  if (e) {
    cudaMemset(engine().dev_err, 0, sizeof(long long));
    if (e & kErrCopiesInFlight) {
      // a CTA left with copies that may still land in shared memory a later
      // launch owns: this plan's results and its next executes are not trusted
      plan->unusable = true;
      return fail(ESTL_DEVICE_ERROR,
                  "a bulk-load wait gave up (tile %lld) and its copies in flight did not drain; the plan is unusable",
                  (e & ~kErrCopiesInFlight) - 1);
    }
    return fail(ESTL_TIMEOUT, "a bulk-load wait gave up (tile %lld)", e - 1);
  }
  return ESTL_OK;
}

int64_t estl_plan_launches(estl_plan plan) { return plan ? (int64_t)plan->layout.steps.size() : 0; }

static estl_status check_buffers(const void* in, const void* out) {
  if (!in || !out) return fail(ESTL_INVALID_ARG, "NULL data pointer");
  if (((uintptr_t)in & 7) || ((uintptr_t)out & 7)) return fail(ESTL_INVALID_ARG, "data pointers must be 8-byte aligned");
  if (in == out) return fail(ESTL_INVALID_ARG, "in-place execution is not supported (d_in == d_out)");
  return ESTL_OK;
}

// ---- other host layouts ---------------------------------------------------
// ESTL_LAYOUT_BLOCK_PLANAR: complex element i has its real part at float
// ((i >> 5) << 6) | (i & 31) and its imaginary part 32 floats later
// (PlannarizedComplexArray<5, D>, Complex.h:34-48,97-130).
// ESTL_LAYOUT_SPLIT: all real parts, then all imaginary parts
// (ComplexArray(n, plannar = true), Complex.h:156-192).
__device__ __forceinline__ long long layout_pos(long long i, int elem, int layout, long long total) {
  if (layout == ESTL_LAYOUT_BLOCK_PLANAR) return ((i >> 5) << 6) | ((long long)elem << 5) | (i & 31);
  return (long long)elem * total + i;
}

__global__ void layout_in_kernel(const float* __restrict__ in, cf32* __restrict__ out, long long total, int layout) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    out[i] = cf32{in[layout_pos(i, 0, layout, total)], in[layout_pos(i, 1, layout, total)]};
}

// Writes every element; in the last 32-element block of a block-planar array
// the real slots past the end are zeroed (those imaginary slots lie past the
// array's last used float and are not touched).
__global__ void layout_out_kernel(const cf32* __restrict__ in, float* __restrict__ out, long long total, int layout) {
  const long long end = layout == ESTL_LAYOUT_BLOCK_PLANAR ? ((total + 31) & ~31LL) : total;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < end; i += (long long)gridDim.x * blockDim.x) {
    if (i < total) {
      const cf32 v = in[i];
      out[layout_pos(i, 0, layout, total)] = v.x;
      out[layout_pos(i, 1, layout, total)] = v.y;
    } else {
      out[layout_pos(i, 0, layout, total)] = 0.f;
    }
  }
}

// Floats of a host array in `layout` holding `total` complex elements: up to
// and including the last float any element uses.
static long long layout_floats(int layout, long long total) {
  if (total <= 0) return 0;
  if (layout == ESTL_LAYOUT_BLOCK_PLANAR) return (((total - 1) >> 5) << 6) + 32 + ((total - 1) & 31) + 1;
  return 2 * total;
}

static int layout_grid(long long total) {
  const long long blocks = (total + 255) / 256;
  return (int)std::max(1LL, std::min<long long>(blocks, 152LL * 16));
}

static estl_status launch_layout_in(int layout, const float* src, cf32* dst, long long total, cudaStream_t st) {
  layout_in_kernel<<<layout_grid(total), 256, 0, st>>>(src, dst, total, layout);
  return check_cuda(cudaGetLastError(), "layout conversion (in)");
}

static estl_status launch_layout_out(int layout, const cf32* src, float* dst, long long total, cudaStream_t st) {
  layout_out_kernel<<<layout_grid(total), 256, 0, st>>>(src, dst, total, layout);
  return check_cuda(cudaGetLastError(), "layout conversion (out)");
}

static estl_status pool_event(estl_plan p, cudaEvent_t* e) {
  if (!p->event_pool.empty()) {
    *e = p->event_pool.back();
    p->event_pool.pop_back();
    return ESTL_OK;
  }
  return check_cuda(cudaEventCreate(e), "cudaEventCreate");
}

// Resolves recorded launch events into the per-kind accumulators (blocks
// until the last recorded launch has finished).
static estl_status resolve_profile(estl_plan p) {
  if (p->pending.empty()) return ESTL_OK;
  estl_status s = check_cuda(cudaEventSynchronize(p->pending.back().b), "cudaEventSynchronize");
  if (s != ESTL_OK) return s;
  for (auto& r : p->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, r.a, r.b);
    p->prof_launches[r.kind] += 1;
    p->prof_ms[r.kind] += ms;
    p->prof_bytes[r.kind] += r.bytes;
    p->event_pool.push_back(r.a);
    p->event_pool.push_back(r.b);
  }
  p->pending.clear();
  return ESTL_OK;
}

static estl_status launch_profiled(estl_plan p, const Plan1D& layout, const cf32* in, cf32* out,
                                   cudaStream_t stream) {
  if (p->pending.size() > 65536) {
    estl_status s = resolve_profile(p);
    if (s != ESTL_OK) return s;
  }
  for (const Step& st : layout.steps) {
    Plan1D one = layout;
    one.steps.assign(1, st);
    estl_plan_s::Rec r{st.kind, 16.0 * (double)st.src_len, nullptr, nullptr};
    estl_status s = pool_event(p, &r.a);
    if (s == ESTL_OK) s = pool_event(p, &r.b);
    if (s == ESTL_OK) s = check_cuda(cudaEventRecord(r.a, stream), "cudaEventRecord");
    if (s == ESTL_OK) s = launch_steps(one, in, out, p->scratch, p->sgn, stream);
    if (s == ESTL_OK) s = check_cuda(cudaEventRecord(r.b, stream), "cudaEventRecord");
    if (s != ESTL_OK) return s;
    p->pending.push_back(r);
  }
  return ESTL_OK;
}

// Conversions of the other host layouts around a plan: `src` (layout) ->
// the plan's interleaved input, its interleaved output -> `dst` (layout).
struct LayoutIO {
  int layout;
  const float* src;
  float* dst;
  long long total;  // complex elements
};

static estl_status run_plan_on(estl_plan plan, const Plan1D& layout, const cf32* in, cf32* out,
                               cudaStream_t stream, const LayoutIO* io = nullptr) {
  std::lock_guard<std::mutex> g(plan->mu);
  if (plan->unusable) return fail(ESTL_DEVICE_ERROR, "the plan is unusable (estl_plan_check reported copies in flight)");
  estl_status s;
  // executes that touch device state of the plan (scratch, staging,
  // Bluestein buffers, profiling events) are ordered behind the previous one;
  // a plan without such state (one tile launch in to out) is not
  const bool stateful = layout.scratch_elems > 0 || layout.blue_m > 0 || io || plan->profiling;
  if (stateful && plan->done_recorded) {
    s = check_cuda(cudaStreamWaitEvent(stream, plan->done, 0), "cudaStreamWaitEvent");
    if (s != ESTL_OK) return s;
  }
  if (io) {
    s = launch_layout_in(io->layout, io->src, const_cast<cf32*>(in), io->total, stream);
    if (s != ESTL_OK) return s;
  }
  if (layout.blue_m > 0)
    s = run_bluestein(plan, layout.batch, in, out, stream);
  else if (plan->profiling)
    s = launch_profiled(plan, layout, in, out, stream);
  else
    s = launch_steps(layout, in, out, plan->scratch, plan->sgn, stream);
  if (s != ESTL_OK) return s;
  if (io) {
    s = launch_layout_out(io->layout, out, io->dst, io->total, stream);
    if (s != ESTL_OK) return s;
  }
  if (!stateful) return ESTL_OK;
  s = check_cuda(cudaEventRecord(plan->done, stream), "cudaEventRecord");
  if (s != ESTL_OK) return s;
  plan->done_recorded = true;
  return ESTL_OK;
}

estl_status estl_execute(estl_plan plan, const void* d_in, void* d_out, void* stream) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  s = check_buffers(d_in, d_out);
  if (s != ESTL_OK) return s;
  return run_plan_on(plan, plan->layout, (const cf32*)d_in, (cf32*)d_out, (cudaStream_t)stream);
}

static estl_status host_pipeline_setup(estl_plan p) {
  if (p->host_ready) return ESTL_OK;
  const long long n = p->layout.n, batch = p->layout.batch;
  // ~64 MiB chunks: large enough to reach copy-engine bandwidth, small
  // enough that the copy in, the transform and the copy out overlap.
  long long chunk = std::max(1LL, (64LL << 20) / (8 * n));
  chunk = std::min(chunk, batch);
  std::string err;
  if (!make_plan_like(p->layout, chunk, &p->host_plan_full, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  long long tail = batch % chunk;
  if (tail && !make_plan_like(p->layout, tail, &p->host_plan_tail, &err))
    return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
  if ((size_t)p->host_plan_full.scratch_elems * sizeof(cf32) > p->scratch_bytes)
    return fail(ESTL_DEVICE_ERROR, "chunk plan needs more scratch than the plan holds");
  p->stage_bytes = (size_t)(chunk * n) * sizeof(cf32);
  estl_status s;
  for (int i = 0; i < 2; ++i) {
    s = dev_alloc((void**)&p->din[i], p->stage_bytes, "host pipeline staging");
    if (s != ESTL_OK) return s;
    s = dev_alloc((void**)&p->dout[i], p->stage_bytes, "host pipeline staging");
    if (s != ESTL_OK) return s;
    if ((s = check_cuda(cudaEventCreateWithFlags(&p->ev_h2d[i], cudaEventDisableTiming), "cudaEventCreate")) != ESTL_OK ||
        (s = check_cuda(cudaEventCreateWithFlags(&p->ev_comp[i], cudaEventDisableTiming), "cudaEventCreate")) != ESTL_OK ||
        (s = check_cuda(cudaEventCreateWithFlags(&p->ev_d2h[i], cudaEventDisableTiming), "cudaEventCreate")) != ESTL_OK)
      return s;
  }
  for (int i = 0; i < 3; ++i) {
    s = check_cuda(cudaStreamCreateWithFlags(&p->st[i], cudaStreamNonBlocking), "cudaStreamCreate");
    if (s != ESTL_OK) return s;
  }
  p->host_chunk = chunk;
  p->host_ready = true;
  return ESTL_OK;
}

// The plan of a ramp chunk of `cnt` transforms (made on first use).
static estl_status ramp_chunk(estl_plan p, long long cnt, const Plan1D** lay) {
  auto it = p->ramp.find(cnt);
  if (it == p->ramp.end()) {
    estl_plan_s::RampChunk rc;
    std::string err;
    if (!make_plan_like(p->layout, cnt, &rc.lay, &err)) return fail(ESTL_UNSUPPORTED_SIZE, "%s", err.c_str());
    it = p->ramp.emplace(cnt, rc).first;
  }
  *lay = &it->second.lay;
  return ESTL_OK;
}

// Chunk sizes (transforms) of one host pipeline run: full chunks, opened by
// chunks of 1/8, 1/4 and 1/2 and closed the same way in reverse, so that the
// first copy-in and the last copy-out (which overlap nothing) are short.
static std::vector<long long> host_schedule(long long batch, long long chunk) {
  std::vector<long long> ramp;
  for (long long d : {8LL, 4LL, 2LL})
    if (chunk / d >= 1 && (ramp.empty() || chunk / d != ramp.back())) ramp.push_back(chunk / d);
  std::vector<long long> out;
  long long sum_ramp = 0;
  for (long long r : ramp) sum_ramp += r;
  if (batch < 4 * chunk || ramp.empty()) {  // too short for a steady state: equal chunks
    for (long long b0 = 0; b0 < batch; b0 += chunk) out.push_back(std::min(chunk, batch - b0));
    return out;
  }
  for (long long r : ramp) out.push_back(r);
  long long mid = batch - 2 * sum_ramp;
  for (; mid > 0; mid -= chunk) out.push_back(std::min(chunk, mid));
  for (auto it = ramp.rbegin(); it != ramp.rend(); ++it) out.push_back(*it);
  return out;
}

estl_status estl_execute_host(estl_plan plan, const float* h_in, float* h_out) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  if (plan->unusable) return fail(ESTL_DEVICE_ERROR, "the plan is unusable (estl_plan_check reported copies in flight)");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  s = check_buffers(h_in, h_out);
  if (s != ESTL_OK) return s;
  std::lock_guard<std::mutex> hg(plan->host_mu);
  s = host_pipeline_setup(plan);
  if (s != ESTL_OK) return s;
  const long long n = plan->layout.n, batch = plan->layout.batch, chunk = plan->host_chunk;
  const std::vector<long long> sched = host_schedule(batch, chunk);
  const long long nchunks = (long long)sched.size();
  cudaStream_t sh = plan->st[0], sc = plan->st[1], sd = plan->st[2];
  long long b0 = 0;
  for (long long i = 0; i < nchunks; b0 += sched[(size_t)i], ++i) {
    const int k = (int)(i & 1);
    const long long cnt = sched[(size_t)i];
    const size_t bytes = (size_t)(cnt * n) * sizeof(cf32);
    const Plan1D* layp = &plan->host_plan_full;
    if (cnt != chunk) {
      if (cnt == batch % chunk) {
        layp = &plan->host_plan_tail;
      } else if ((s = ramp_chunk(plan, cnt, &layp)) != ESTL_OK) {
        return s;
      }
    }
    const Plan1D& lay = *layp;
    if (i >= 2 && (s = check_cuda(cudaStreamWaitEvent(sh, plan->ev_comp[k], 0), "wait")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaMemcpyAsync(plan->din[k], h_in + 2 * b0 * n, bytes, cudaMemcpyHostToDevice, sh),
                        "cudaMemcpyAsync(H2D)")) != ESTL_OK)
      return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_h2d[k], sh), "record")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaStreamWaitEvent(sc, plan->ev_h2d[k], 0), "wait")) != ESTL_OK) return s;
    if (i >= 2 && (s = check_cuda(cudaStreamWaitEvent(sc, plan->ev_d2h[k], 0), "wait")) != ESTL_OK) return s;
    if ((s = run_plan_on(plan, lay, plan->din[k], plan->dout[k], sc)) != ESTL_OK) return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_comp[k], sc), "record")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaStreamWaitEvent(sd, plan->ev_comp[k], 0), "wait")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaMemcpyAsync(h_out + 2 * b0 * n, plan->dout[k], bytes, cudaMemcpyDeviceToHost, sd),
                        "cudaMemcpyAsync(D2H)")) != ESTL_OK)
      return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_d2h[k], sd), "record")) != ESTL_OK) return s;
  }
  return check_cuda(cudaStreamSynchronize(sd), "cudaStreamSynchronize");
}

estl_status estl_execute_layout(estl_plan plan, int layout, const float* d_in, float* d_out, void* stream) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  if (layout == ESTL_LAYOUT_INTERLEAVED) return estl_execute(plan, d_in, d_out, stream);
  if (layout != ESTL_LAYOUT_BLOCK_PLANAR && layout != ESTL_LAYOUT_SPLIT)
    return fail(ESTL_INVALID_ARG, "unknown layout %d", layout);
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (!d_in || !d_out || ((uintptr_t)d_in & 3) || ((uintptr_t)d_out & 3) || d_in == d_out)
    return fail(ESTL_INVALID_ARG, "need distinct, 4-byte aligned device buffers");
  const long long total = plan->layout.n * plan->layout.batch;
  {
    std::lock_guard<std::mutex> g(plan->mu);
    if (!plan->lay_in) {
      const size_t bytes = (size_t)total * sizeof(cf32);
      s = dev_alloc((void**)&plan->lay_in, bytes, "layout staging");
      if (s == ESTL_OK) s = dev_alloc((void**)&plan->lay_out, bytes, "layout staging");
      if (s != ESTL_OK) {
        dev_free(plan->lay_in, bytes);
        plan->lay_in = nullptr;
        return s;
      }
      plan->lay_bytes = bytes;
    }
  }
  LayoutIO io{layout, d_in, d_out, total};
  return run_plan_on(plan, plan->layout, plan->lay_in, plan->lay_out, (cudaStream_t)stream, &io);
}

estl_status estl_execute_host_layout(estl_plan plan, int layout, const float* h_in, float* h_out) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  if (layout == ESTL_LAYOUT_INTERLEAVED) return estl_execute_host(plan, h_in, h_out);
  if (layout != ESTL_LAYOUT_BLOCK_PLANAR && layout != ESTL_LAYOUT_SPLIT)
    return fail(ESTL_INVALID_ARG, "unknown layout %d", layout);
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (!h_in || !h_out || h_in == h_out) return fail(ESTL_INVALID_ARG, "need distinct host buffers");
  std::lock_guard<std::mutex> hg(plan->host_mu);
  s = host_pipeline_setup(plan);
  if (s != ESTL_OK) return s;
  const long long n = plan->layout.n, batch = plan->layout.batch, chunk = plan->host_chunk, total = n * batch;
  if (!plan->hlay_in[0]) {
    // raw-layout staging of one chunk (chunk * n is 0 mod 32 or the whole batch, so
    // every block-planar chunk starts on a 32-element block)
    const size_t bytes = (size_t)std::max(layout_floats(ESTL_LAYOUT_BLOCK_PLANAR, chunk * n), 2 * chunk * n) * 4;
    for (int k = 0; k < 2 && s == ESTL_OK; ++k) {
      s = dev_alloc((void**)&plan->hlay_in[k], bytes, "layout staging");
      if (s == ESTL_OK) s = dev_alloc((void**)&plan->hlay_out[k], bytes, "layout staging");
    }
    plan->hlay_bytes = bytes;
    if (s != ESTL_OK) return s;
  }
  const long long nchunks = (batch + chunk - 1) / chunk;
  cudaStream_t sh = plan->st[0], sc = plan->st[1], sd = plan->st[2];
  for (long long i = 0; i < nchunks; ++i) {
    const int k = (int)(i & 1);
    const long long b0 = i * chunk, cnt = std::min(chunk, batch - b0), e0 = b0 * n, ce = cnt * n;
    const Plan1D& lay = cnt == chunk ? plan->host_plan_full : plan->host_plan_tail;
    if (i >= 2 && (s = check_cuda(cudaStreamWaitEvent(sh, plan->ev_comp[k], 0), "wait")) != ESTL_OK) return s;
    if (layout == ESTL_LAYOUT_BLOCK_PLANAR) {
      s = check_cuda(cudaMemcpyAsync(plan->hlay_in[k], h_in + 2 * e0, (size_t)layout_floats(layout, ce) * 4,
                                     cudaMemcpyHostToDevice, sh),
                     "cudaMemcpyAsync(H2D)");
    } else {  // split: the chunk's real parts, then its imaginary parts
      s = check_cuda(cudaMemcpyAsync(plan->hlay_in[k], h_in + e0, (size_t)ce * 4, cudaMemcpyHostToDevice, sh),
                     "cudaMemcpyAsync(H2D)");
      if (s == ESTL_OK)
        s = check_cuda(cudaMemcpyAsync(plan->hlay_in[k] + ce, h_in + total + e0, (size_t)ce * 4,
                                       cudaMemcpyHostToDevice, sh),
                       "cudaMemcpyAsync(H2D)");
    }
    if (s != ESTL_OK) return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_h2d[k], sh), "record")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaStreamWaitEvent(sc, plan->ev_h2d[k], 0), "wait")) != ESTL_OK) return s;
    if (i >= 2 && (s = check_cuda(cudaStreamWaitEvent(sc, plan->ev_d2h[k], 0), "wait")) != ESTL_OK) return s;
    LayoutIO io{layout, plan->hlay_in[k], plan->hlay_out[k], ce};
    if ((s = run_plan_on(plan, lay, plan->din[k], plan->dout[k], sc, &io)) != ESTL_OK) return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_comp[k], sc), "record")) != ESTL_OK) return s;
    if ((s = check_cuda(cudaStreamWaitEvent(sd, plan->ev_comp[k], 0), "wait")) != ESTL_OK) return s;
    if (layout == ESTL_LAYOUT_BLOCK_PLANAR) {
      s = check_cuda(cudaMemcpyAsync(h_out + 2 * e0, plan->hlay_out[k], (size_t)layout_floats(layout, ce) * 4,
                                     cudaMemcpyDeviceToHost, sd),
                     "cudaMemcpyAsync(D2H)");
    } else {
      s = check_cuda(cudaMemcpyAsync(h_out + e0, plan->hlay_out[k], (size_t)ce * 4, cudaMemcpyDeviceToHost, sd),
                     "cudaMemcpyAsync(D2H)");
      if (s == ESTL_OK)
        s = check_cuda(cudaMemcpyAsync(h_out + total + e0, plan->hlay_out[k] + ce, (size_t)ce * 4,
                                       cudaMemcpyDeviceToHost, sd),
                       "cudaMemcpyAsync(D2H)");
    }
    if (s != ESTL_OK) return s;
    if ((s = check_cuda(cudaEventRecord(plan->ev_d2h[k], sd), "record")) != ESTL_OK) return s;
  }
  return check_cuda(cudaStreamSynchronize(sd), "cudaStreamSynchronize");
}

int64_t estl_layout_floats(int layout, int64_t total) {
  if (layout == ESTL_LAYOUT_INTERLEAVED || layout == ESTL_LAYOUT_SPLIT) return total > 0 ? 2 * total : 0;
  if (layout == ESTL_LAYOUT_BLOCK_PLANAR) return layout_floats(layout, total);
  return -1;
}

estl_status estl_plan_set_profiling(estl_plan plan, int enable) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> g(plan->mu);
  estl_status s = resolve_profile(plan);
  if (s != ESTL_OK) return s;
  plan->profiling = enable != 0;
  for (int k = 0; k < kStepKinds; ++k) {
    plan->prof_launches[k] = 0;
    plan->prof_ms[k] = 0;
    plan->prof_bytes[k] = 0;
  }
  return ESTL_OK;
}

estl_status estl_plan_kernel_stats(estl_plan plan, int64_t* launches, double* total_ms, double* bytes) {
  if (!plan) return fail(ESTL_INVALID_ARG, "NULL plan");
  std::lock_guard<std::mutex> g(plan->mu);
  estl_status s = resolve_profile(plan);
  if (s != ESTL_OK) return s;
  for (int k = 0; k < kStepKinds; ++k) {
    if (launches) launches[k] = plan->prof_launches[k];
    if (total_ms) total_ms[k] = plan->prof_ms[k];
    if (bytes) bytes[k] = plan->prof_bytes[k];
  }
  return ESTL_OK;
}

estl_status estl_host_register(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return fail(ESTL_INVALID_ARG, "NULL pointer or zero size");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  return check_cuda(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault), "cudaHostRegister");
}

estl_status estl_host_unregister(void* ptr) {
  if (!ptr) return fail(ESTL_INVALID_ARG, "NULL pointer");
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  return check_cuda(cudaHostUnregister(ptr), "cudaHostUnregister");
}

estl_status estl_memory_usage(size_t* used_bytes, size_t* budget_bytes) {
  Engine& E = engine();
  if (used_bytes) *used_bytes = E.used.load();
  if (budget_bytes) *budget_bytes = E.budget;
  return ESTL_OK;
}

}  // extern "C"
