/* Interface-compatible stand-in for ESTL's FFT.h (test infrastructure; see
 * Complex.h in this directory for why it exists).  Keeps the plugin API the
 * backends implement and the drivers call: FFT<D> (FFT.h:19-36),
 * FFTFactory<D> / FFTFactorySpecific<C> (FFT.h:38-52) and FFT2D<D>
 * (FFT.h:54-84, a row pass then a column pass of batch-1 1D transforms). */
#ifndef FFT_H
#define FFT_H

#include <string>

#include "Complex.h"
#include "DataInterface.h"

typedef std::string streng;

template <class D>
class FFT {
 public:
  typedef D DataType;
  DataInterface<D>* dataInterface;
  int size, batchCount;
  FFT(int n, int batch) : dataInterface(NULL), size(n), batchCount(batch) {}
  virtual ~FFT() { delete dataInterface; }
  static int getMaxBatchSize(int) { return 1; }
  void setData(int index, Complex<D> v, int batchIndex = 0) { dataInterface->setElement(batchIndex * size + index, v); }
  Complex<D> getData(int index, int batchIndex = 0) { return dataInterface->getElement(batchIndex * size + index); }
  virtual void execute() = 0;
};

template <class D>
class FFTFactory {
 public:
  virtual ~FFTFactory() {}
  virtual streng getName() = 0;
  virtual int getVersion() { return 0; }
  virtual FFT<D>* newFFT(int n, bool forward = true, int batchSize = 1) = 0;
  virtual int getMaxBatchSize(int) { return 1; }
};

template <class C>
class FFTFactorySpecific : public FFTFactory<typename C::DataType> {
  typedef typename C::DataType D;

 public:
  streng getName() { return C::getName(); }
  int getMaxBatchSize(int n) { return C::getMaxBatchSize(n); }
  FFT<D>* newFFT(int n, bool forward = true, int batchSize = 1) { return new C(n, forward, batchSize); }
};

template <class D>
class FFT2D {
 public:
  Complex<D>* data;
  int xDim, yDim;
  FFTFactory<D>* fftFactory;
  bool forward;
  FFT2D(int x, int y, FFTFactory<D>* f, bool fwd = true) : xDim(x), yDim(y), fftFactory(f), forward(fwd) {
    data = new Complex<D>[(size_t)x * y];
  }
  virtual ~FFT2D() { delete[] data; }
  virtual void execute() {
    FFT<D>* fx = fftFactory->newFFT(xDim, forward);
    for (int y = 0; y < yDim; ++y) {
      for (int x = 0; x < xDim; ++x) fx->setData(x, data[y * xDim + x]);
      fx->execute();
      for (int x = 0; x < xDim; ++x) data[y * xDim + x] = fx->getData(x);
    }
    delete fx;
    FFT<D>* fy = fftFactory->newFFT(yDim, forward);
    for (int x = 0; x < xDim; ++x) {
      for (int y = 0; y < yDim; ++y) fy->setData(y, data[y * xDim + x]);
      fy->execute();
      for (int y = 0; y < yDim; ++y) data[y * xDim + x] = fy->getData(y);
    }
    delete fy;
  }
};

#endif
