// conv2d.cu — 2D FFT convolution (Convolution2D_FFT, Convolution.h:95-148):
// kernel registry, plan and C ABI.  The kernels are in conv2d_core.cuh.
#include <algorithm>
#include <climits>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "conv2d_core.cuh"
#include "engine.h"

namespace estl {

template <class K>
__global__ void __launch_bounds__(K::NT, K::MIN_BLOCKS) conv2d_kernel(Conv2dArgs a) {
  extern __shared__ float2 estl_conv2d_smem[];
  pdl_enter();
  K::run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_conv2d_smem));
}

namespace {

constexpr long long kConv2dMaxSmemBytes = 227 * 1024;

struct Conv2dKernelDesc {
  int col;  // 0 row kernel, 1 column kernel
  int logm, loge, logc;
  int nthreads, smem_bytes;
  const void* fn;
  bool attr_set;
};

template <class K>
Conv2dKernelDesc c2desc(int col, int m, int e, int c) {
  return Conv2dKernelDesc{col, m, e, c, K::NT, (int)(K::SMEM_ELEMS * sizeof(cf32)),
                          reinterpret_cast<const void*>(&conv2d_kernel<K>), false};
}

#define ESTL_X_C2ROW(M, E, C) \
  static_assert(Conv2dRowKernel<M, E, 4, C>::SMEM_ELEMS * 8 <= kConv2dMaxSmemBytes, "2D row tile too large");
#define ESTL_X_C2COL(M, E, C) \
  static_assert(Conv2dColKernel<M, E, 4, C>::SMEM_ELEMS * 8 <= kConv2dMaxSmemBytes, "2D column tile too large");
#include "conv2d_list.inc"

std::vector<Conv2dKernelDesc>& conv2d_table() {
  static std::vector<Conv2dKernelDesc> t = [] {
    std::vector<Conv2dKernelDesc> v;
#define ESTL_X_C2ROW(M, E, C) v.push_back(c2desc<Conv2dRowKernel<M, E, 4, C>>(0, M, E, C));
#define ESTL_X_C2COL(M, E, C) v.push_back(c2desc<Conv2dColKernel<M, E, 4, C>>(1, M, E, C));
#include "conv2d_list.inc"
    return v;
  }();
  return t;
}

std::mutex g_conv2d_attr_mu;

// The row tile of a padded width, or the widest column tile of a padded
// height that does not exceed the padded width.
estl_status conv2d_pick(int col, int logm, int logw, Conv2dKernelDesc** out) {
  Conv2dKernelDesc* best = nullptr;
  for (Conv2dKernelDesc& d : conv2d_table())
    if (d.col == col && d.logm == logm && (!col || d.logc <= logw) && (!best || d.logc > best->logc)) best = &d;
  if (!best) return fail(ESTL_UNSUPPORTED_SIZE, "no 2D convolution tile for 2^%d points (%s)", logm, col ? "columns" : "rows");
  if (!best->attr_set) {
    std::lock_guard<std::mutex> g(g_conv2d_attr_mu);
    if (!best->attr_set) {
      estl_status s = check_cuda(cudaFuncSetAttribute(best->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, best->smem_bytes),
                                 "cudaFuncSetAttribute(conv2d)");
      if (s != ESTL_OK) return s;
      best->attr_set = true;
    }
  }
  *out = best;
  return ESTL_OK;
}

estl_status conv2d_launch(const Conv2dKernelDesc* d, const Conv2dArgs& a, cudaStream_t stream) {
  const long long grid = conv2d_grid(d->col != 0, d->logc, a);
  if (grid < 1) return ESTL_OK;
  if (grid > INT_MAX) return fail(ESTL_UNSUPPORTED_SIZE, "2D convolution grid of %lld CTAs", grid);
  Conv2dArgs b = a;
  void* args[] = {&b};
  return launch_pdl(d->fn, grid, d->nthreads, args, d->smem_bytes, stream, "cudaLaunchKernelEx(conv2d)");
}

}  // namespace
}  // namespace estl

using namespace estl;

struct estl_conv2d_plan_s {
  Conv2dGeom g;
  long long w = 0, h = 0, kw = 0, kh = 0, count = 0;
  int flags = 0;
  Conv2dKernelDesc* row = nullptr;
  Conv2dKernelDesc* col = nullptr;
  cf32* spec = nullptr;
  size_t spec_bytes = 0;
  cf32* work = nullptr;
  size_t work_bytes = 0;
  bool filter_set = false;
};

extern "C" {

estl_status estl_conv2d_output_size(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int flags,
                                    int64_t* out_width, int64_t* out_height) {
  Conv2dGeom g;
  if (!conv2d_geometry(width, height, kwidth, kheight, (flags & ESTL_CONV_REFERENCE_COMPAT) != 0, &g))
    return fail(ESTL_INVALID_ARG, "2D convolution sizes must be in [1, 2^20] (got %lld x %lld, filter %lld x %lld)",
                (long long)width, (long long)height, (long long)kwidth, (long long)kheight);
  if (out_width) *out_width = g.out_w;
  if (out_height) *out_height = g.out_h;
  return ok();
}

estl_status estl_conv2d_plan_create(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int64_t count,
                                    int flags, estl_conv2d_plan* plan) {
  if (!plan) return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_create: null plan pointer");
  *plan = nullptr;
  estl_status s = require_init();
  if (s != ESTL_OK) return s;
  if (flags & ~(ESTL_CONV_CORRELATE | ESTL_CONV_REFERENCE_COMPAT))
    return fail(ESTL_INVALID_ARG, "2D convolution flags: CORRELATE and REFERENCE_COMPAT only, FP32 (got 0x%x)", flags);
  if (count < 1) return fail(ESTL_INVALID_ARG, "2D convolution needs count >= 1 (got %lld)", (long long)count);
  Conv2dGeom g;
  if (!conv2d_geometry(width, height, kwidth, kheight, (flags & ESTL_CONV_REFERENCE_COMPAT) != 0, &g))
    return fail(ESTL_INVALID_ARG, "2D convolution sizes must be in [1, 2^20] (got %lld x %lld, filter %lld x %lld)",
                (long long)width, (long long)height, (long long)kwidth, (long long)kheight);
  if (!conv2d_supported(g))
    return fail(ESTL_UNSUPPORTED_SIZE,
                "2D convolution pads to 2^%d x 2^%d: needs width <= 2^14, height <= 2^12 and at most 2^26 points",
                g.logw, g.logh);
  std::unique_ptr<estl_conv2d_plan_s> p(new estl_conv2d_plan_s);
  p->g = g;
  p->w = width;
  p->h = height;
  p->kw = kwidth;
  p->kh = kheight;
  p->count = count;
  p->flags = flags;
  s = conv2d_pick(0, g.logw, g.logw, &p->row);
  if (s == ESTL_OK) s = conv2d_pick(1, g.logh, g.logw, &p->col);
  if (s != ESTL_OK) return s;
  const long long pts = 1LL << (g.logw + g.logh);
  p->spec_bytes = (size_t)pts * sizeof(cf32);
  if ((unsigned long long)count > (unsigned long long)(LLONG_MAX / 8) / (unsigned long long)pts)
    return fail(ESTL_OUT_OF_MEMORY, "2D convolution work array of %lld x %lld points", (long long)count, pts);
  p->work_bytes = (size_t)(count * pts) * sizeof(cf32);
  s = dev_alloc((void**)&p->spec, p->spec_bytes, "2D convolution filter spectrum");
  if (s != ESTL_OK) return s;
  s = dev_alloc((void**)&p->work, p->work_bytes, "2D convolution work array");
  if (s != ESTL_OK) {
    dev_free(p->spec, p->spec_bytes);
    return s;
  }
  *plan = p.release();
  return ok();
}

// The filter spectrum: passes 1 and 2 in spectrum mode on the filter, scaled
// by 1 / (Pw Ph) and conjugated for correlation.
estl_status estl_conv2d_plan_set_filter(estl_conv2d_plan p, const float* d_filter, void* stream) {
  if (!p || !d_filter) return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_set_filter: null argument");
  if ((uintptr_t)d_filter & 3) return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_set_filter: filter must be 4-byte aligned");
  Engine& E = engine();
  const cudaStream_t st = (cudaStream_t)stream;
  Conv2dArgs a = conv2d_filter_args(p->g, p->kw, p->kh, (p->flags & ESTL_CONV_REFERENCE_COMPAT) != 0,
                                    (p->flags & ESTL_CONV_CORRELATE) != 0, d_filter, p->spec, E.bank, kBankSize);
  estl_status s = conv2d_launch(p->row, a, st);
  if (s != ESTL_OK) return s;
  a.mode = 1;
  s = conv2d_launch(p->col, a, st);
  if (s != ESTL_OK) return s;
  p->filter_set = true;
  return ok();
}

estl_status estl_conv2d_plan_execute(estl_conv2d_plan p, const float* d_images, float* d_out, void* stream) {
  if (!p || !d_images || !d_out) return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_execute: null argument");
  if (!p->filter_set) return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_execute: set the filter first");
  if (((uintptr_t)d_images | (uintptr_t)d_out) & 3)
    return fail(ESTL_INVALID_ARG, "estl_conv2d_plan_execute: buffers must be 4-byte aligned");
  Engine& E = engine();
  const cudaStream_t st = (cudaStream_t)stream;
  Conv2dArgs a = conv2d_exec_args(p->g, p->w, p->h, p->count, (p->flags & ESTL_CONV_REFERENCE_COMPAT) != 0, d_images,
                                  p->work, p->spec, d_out, E.bank, kBankSize);
  estl_status s = conv2d_launch(p->row, a, st);
  if (s != ESTL_OK) return s;
  s = conv2d_launch(p->col, a, st);
  if (s != ESTL_OK) return s;
  a.mode = 1;
  s = conv2d_launch(p->row, a, st);
  if (s != ESTL_OK) return s;
  return ok();
}

// One image, host buffers, blocking: the call Convolution2D_FFT::convolve
// makes (Convolution.h:95-148), for the C++ plugin Convolution2D_FFT_CUDA.
estl_status estl_conv2d_host(int64_t width, int64_t height, int64_t kwidth, int64_t kheight, int flags,
                             const float* h_image, const float* h_kernel, float* h_out) {
  if (!h_image || !h_kernel || !h_out) return fail(ESTL_INVALID_ARG, "estl_conv2d_host: null argument");
  estl_conv2d_plan p = nullptr;
  estl_status s = estl_conv2d_plan_create(width, height, kwidth, kheight, 1, flags, &p);
  if (s != ESTL_OK) return s;
  const size_t in_b = (size_t)(width * height) * sizeof(float), k_b = (size_t)(kwidth * kheight) * sizeof(float);
  const size_t out_b = (size_t)p->g.out_w * (size_t)p->g.out_h * sizeof(float);
  float *d_in = nullptr, *d_k = nullptr, *d_out = nullptr;
  s = dev_alloc((void**)&d_in, in_b, "2D convolution image");
  if (s == ESTL_OK) s = dev_alloc((void**)&d_k, k_b, "2D convolution filter");
  if (s == ESTL_OK) s = dev_alloc((void**)&d_out, out_b, "2D convolution output");
  if (s == ESTL_OK) s = check_cuda(cudaMemcpy(d_in, h_image, in_b, cudaMemcpyHostToDevice), "cudaMemcpy(image)");
  if (s == ESTL_OK) s = check_cuda(cudaMemcpy(d_k, h_kernel, k_b, cudaMemcpyHostToDevice), "cudaMemcpy(filter)");
  if (s == ESTL_OK) s = estl_conv2d_plan_set_filter(p, d_k, nullptr);
  if (s == ESTL_OK) s = estl_conv2d_plan_execute(p, d_in, d_out, nullptr);
  if (s == ESTL_OK) s = check_cuda(cudaMemcpy(h_out, d_out, out_b, cudaMemcpyDeviceToHost), "cudaMemcpy(output)");
  const estl_status keep = s;
  const std::string msg = keep == ESTL_OK ? std::string() : std::string(estl_last_error());
  cudaDeviceSynchronize();
  if (d_in) dev_free(d_in, in_b);
  if (d_k) dev_free(d_k, k_b);
  if (d_out) dev_free(d_out, out_b);
  estl_conv2d_plan_destroy(p);
  if (keep != ESTL_OK) return fail(keep, "%s", msg.c_str());
  return ok();
}

int64_t estl_conv2d_plan_launches(estl_conv2d_plan p) { return p ? 3 : 0; }

estl_status estl_conv2d_plan_destroy(estl_conv2d_plan p) {
  if (!p) return ok();
  cudaDeviceSynchronize();
  dev_free(p->spec, p->spec_bytes);
  dev_free(p->work, p->work_bytes);
  delete p;
  return ok();
}

}  // extern "C"
