/* FFT_CUDA.h — ESTL backend plugin for the GB300 FFT engine.
 *
 * FFT_CUDA<D> is an FFT<D> (FFT.h:19-36) like FFT_FFTW3<D> (FFT_FFTW3.h:16-34)
 * and FFT_OpenCL_Contiguous<D> (FFT_OpenCL_Contiguous.h:26-192), so it drops
 * into every place the reference creates a backend through a factory:
 *
 *   factories.push_back(new FFTFactorySpecific<FFT_CUDA<T> >());   // tests/Test.cpp:196-200
 *   FFTFactory<S>* f = new FFTFactorySpecific<FFT_CUDA<S> >();      // Convolution.h:101
 *
 * It uses the interleaved host layout of FFT_FFTW3
 * (SplitInterleavedDataInterface(n*batch, false), FFT_FFTW3.h:24), pins those
 * host arrays once, and executes through the C ABI (estl_cuda.h): copy in,
 * all passes on the device, copy out, with the copies and the transform
 * pipelined.  Backward transforms are exact for every transform of the batch.
 *
 * The per-kernel timers keep the member names of OpenCLAlgorithm
 * (uOpenCL.h:281-282, 339-340) on the GpuAlgorithm mix-in, so a driver written
 * like tests/Test.cpp:56,86-99 reads them after dynamic_cast<GpuAlgorithm*>.
 *
 * Errors: C ABI status codes become EstlException (the reference throws
 * CLException from xCLErr, uOpenCL.h:21-55).
 *
 * Include after ESTL's FFT.h (or an interface-compatible copy of it).
 */
#ifndef FFT_CUDA_H
#define FFT_CUDA_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <exception>
#include <string>
#include <vector>

#include "FFT.h"
#include "estl_cuda.h"

class EstlException : public std::exception {
 public:
  EstlException(estl_status s, const std::string& where)
      : status(s), msg(std::string("[") + estl_status_string(s) + "] " + where + ": " + estl_last_error()) {}
  virtual const char* what() const throw() { return msg.c_str(); }
  virtual ~EstlException() throw() {}
  estl_status status;

 private:
  std::string msg;
};

inline void estlCheck(estl_status s, const char* where) {
  if (s != ESTL_OK) throw EstlException(s, where);
}

/* Default timer with the interface of ESTL's Timer (tests/Timer.h:47-116);
 * ESTL's own Timer is used instead when tests/Timer.h was included first. */
class EstlHostTimer {
 public:
  EstlHostTimer() : totalTime(0), runs(0) {}
  void addRun(double t) {
    totalTime += t;
    runs++;
  }
  double getTotalTime() { return totalTime; }
  double getAverageTime() { return runs ? totalTime / runs : 0; }
  int getRuns() { return runs; }

 private:
  double totalTime;
  int runs;
};

#ifdef TIMER_H
typedef Timer EstlTimerType;
#else
typedef EstlHostTimer EstlTimerType;
#endif

/* Instrumentation contract of OpenCLAlgorithm (uOpenCL.h:275-348). */
class GpuAlgorithm {
 public:
  EstlTimerType *timerComputation, *timerTotal;
  std::vector<EstlTimerType> kernelTimers;
  GpuAlgorithm() : timerComputation(NULL), timerTotal(NULL) {}
  virtual double getTotalComputationFlops(int kernel) { return 0; }
  virtual std::string getKernelInfo(int kernel) { return ""; }
  virtual ~GpuAlgorithm() {}

  static void ensureInit() {
    const char* dev = getenv("ESTL_DEVICE");
    estlCheck(estl_init(dev ? atoi(dev) : 0, 0), "estl_init");
  }
};

/* Host layout of a DataInterface type: SplitInterleavedDataInterface(n,
 * false) is interleaved (the FFT_FFTW3 layout, FFT_FFTW3.h:24);
 * PlannarizedDataInterface is block-planar (the FFT_OpenCL_Contiguous
 * layout, FFT_OpenCL_Contiguous.h:28). */
template <class DI>
struct EstlLayoutOf {
  enum { value = ESTL_LAYOUT_INTERLEAVED };
  static DI* make(int n) { return new DI(n, false); }
};
template <class D>
struct EstlLayoutOf<PlannarizedDataInterface<D> > {
  enum { value = ESTL_LAYOUT_BLOCK_PLANAR };
  static PlannarizedDataInterface<D>* make(int n) { return new PlannarizedDataInterface<D>(n); }
};

/* FFT_CUDA<D> keeps FFT_FFTW3's interleaved host arrays;
 * FFT_CUDA<D, PlannarizedDataInterface<D> > keeps FFT_OpenCL_Contiguous's
 * block-planar ones, so it replaces that backend with the same dataInterface
 * type. */
template <class D, class DI = SplitInterleavedDataInterface<D> >
class FFT_CUDA : public FFT<D>, public GpuAlgorithm {
 public:
  typedef DI DataInterfaceType;

  static streng getName() { return "GB300 CUDA FFT"; }

  /* FFT_OpenCL_Contiguous::getMaxBatchSize (FFT_OpenCL_Contiguous.h:43-44) against the HBM budget. */
  static int getMaxBatchSize(int n) {
    ensureInit();
    int64_t b = estl_max_batch(n);
    return b > 2147483647 ? 2147483647 : (int)b;
  }

  FFT_CUDA(int n, bool forward = true, int iBatchCount = 1)
      : FFT<D>(n, iBatchCount), plan(NULL), registered(false) {
    typedef char only_float_is_supported[(sizeof(D) == sizeof(float)) ? 1 : -1];
    (void)sizeof(only_float_is_supported);
    this->dataInterface = arrays = EstlLayoutOf<DI>::make(this->batchCount * this->size);
    ensureInit();
    estlCheck(estl_plan_create(n, iBatchCount, forward ? ESTL_FORWARD : ESTL_BACKWARD, ESTL_PREC_FP32, &plan),
              "estl_plan_create");
    estlCheck(estl_plan_set_profiling(plan, 1), "estl_plan_set_profiling");
    char desc[1024];
    estl_plan_describe(plan, desc, sizeof desc);
    describe = desc;
    kinds.clear();
    if (describe.find("\"single\"") != std::string::npos) kinds.push_back(0);
    if (describe.find("\"col\"") != std::string::npos) kinds.push_back(1);
    if (describe.find("\"row\"") != std::string::npos) kinds.push_back(2);
    if (describe.find("\"copy\"") != std::string::npos) kinds.push_back(3);
    if (describe.find("\"stream\"") != std::string::npos) kinds.push_back(4);
    if (describe.find("\"column\"") != std::string::npos) kinds.push_back(5);
    kernelTimers.resize(kinds.size());
    const size_t bytes =
        sizeof(D) * (size_t)estl_layout_floats(EstlLayoutOf<DI>::value, (int64_t)this->size * this->batchCount);
    registered = estl_host_register(arrays->in->getData(), bytes) == ESTL_OK &&
                 estl_host_register(arrays->out->getData(), bytes) == ESTL_OK;
    for (int k = 0; k < ESTL_KERNEL_KINDS; ++k) lastMs[k] = 0;
  }

  virtual double getTotalComputationFlops(int kernel) {
    double lg = log((double)this->size) / log(2.0), part = lg;
    int logn = (int)(lg + 0.5);
    if (kinds.size() == 2) part = (kernel == 0) ? (double)(logn / 2) : (double)(logn - logn / 2);
    return 5.0 * this->size * part * this->batchCount;
  }

  virtual std::string getKernelInfo(int kernel) {
    static const char* names[] = {"tile", "column", "row", "copy", "unused", "2D column"};
    return (kernel >= 0 && kernel < (int)kinds.size()) ? names[kinds[kernel]] : "";
  }

  /* FFT<D>::execute: the result is in the data interface's output array. */
  virtual void execute() {
    estlCheck(estl_execute_host_layout(plan, EstlLayoutOf<DI>::value, arrays->in->getData(), arrays->out->getData()),
              "estl_execute_host_layout");
    int64_t launches[ESTL_KERNEL_KINDS];
    double ms[ESTL_KERNEL_KINDS], bytes[ESTL_KERNEL_KINDS];
    estlCheck(estl_plan_kernel_stats(plan, launches, ms, bytes), "estl_plan_kernel_stats");
    double total = 0;
    for (size_t i = 0; i < kinds.size(); ++i) {
      double d = ms[kinds[i]] - lastMs[kinds[i]];
      kernelTimers[i].addRun(1e-3 * d);
      total += d;
    }
    for (int k = 0; k < ESTL_KERNEL_KINDS; ++k) lastMs[k] = ms[k];
    if (timerComputation) timerComputation->addRun(1e-3 * total);
  }

  const std::string& planDescription() const { return describe; }

  virtual ~FFT_CUDA() {
    if (registered) {
      estl_host_unregister(arrays->in->getData());
      estl_host_unregister(arrays->out->getData());
    }
    if (plan) estl_plan_destroy(plan);
  }

 private:
  DataInterfaceType* arrays;
  estl_plan plan;
  bool registered;
  std::string describe;
  std::vector<int> kinds;
  double lastMs[ESTL_KERNEL_KINDS];
};

/* FFT2D_CUDA<D> is an FFT2D<D> (FFT.h:54-84): the same `data` array of
 * xDim * yDim Complex<D> (row-major, x fastest) and the same in-place
 * execute(), which the reference runs as one FFT object per row and per
 * column with per-element copies.  Here execute() is one 2D plan
 * (estl_plan2d_create): row FFTs and column FFTs on the device, the array
 * copied in and out once.  Convolution2D_FFT (Convolution.h:102-104) builds
 * its three FFT2D objects this way when it constructs FFT2D_CUDA instead. */
template <class D>
class FFT2D_CUDA : public FFT2D<D> {
 public:
  FFT2D_CUDA(int iXDim, int iYDim, bool iForward = true)
      : FFT2D<D>(iXDim, iYDim, NULL, iForward), plan(NULL), out((size_t)iXDim * iYDim) {
    typedef char only_float_is_supported[(sizeof(D) == sizeof(float) && sizeof(Complex<D>) == 2 * sizeof(D)) ? 1 : -1];
    (void)sizeof(only_float_is_supported);
    GpuAlgorithm::ensureInit();
    estlCheck(estl_plan2d_create(iXDim, iYDim, 1, iForward ? ESTL_FORWARD : ESTL_BACKWARD, ESTL_PREC_FP32, &plan),
              "estl_plan2d_create");
  }

  virtual void execute() {
    estlCheck(estl_execute_host(plan, reinterpret_cast<const float*>(this->data), reinterpret_cast<float*>(&out[0])),
              "estl_execute_host");
    for (size_t q = 0; q < out.size(); ++q) this->data[q] = out[q];
  }

  virtual ~FFT2D_CUDA() {
    if (plan) estl_plan_destroy(plan);
  }

 private:
  estl_plan plan;
  std::vector<Complex<D> > out;
};

#endif  // FFT_CUDA_H
