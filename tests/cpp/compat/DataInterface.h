/* Interface-compatible stand-in for ESTL's DataInterface.h (test
 * infrastructure; see Complex.h in this directory for why it exists).
 * Keeps DataInterface<D>, ArrayDataInterface<D,A> and
 * SplitInterleavedDataInterface<D> (DataInterface.h:6-45). */
#ifndef DATAINTERFACE_H
#define DATAINTERFACE_H

#include "Complex.h"

template <class D>
class DataInterface {
 public:
  virtual void setElement(int index, Complex<D> value, int batchIndex = 0) = 0;
  virtual Complex<D> getElement(int index, int batchIndex = 0) = 0;
  virtual ~DataInterface() {}
};

template <class D, class A>
class ArrayDataInterface : public DataInterface<D> {
 protected:
  int size;

 public:
  A *in, *out;
  explicit ArrayDataInterface(int n) : size(n), in(NULL), out(NULL) {}
  virtual ~ArrayDataInterface() {
    delete in;
    delete out;
  }
  void setElement(int index, Complex<D> v, int batchIndex = 0) { in->setElement(batchIndex * size + index, v); }
  Complex<D> getElement(int index, int batchIndex = 0) { return out->getElement(batchIndex * size + index); }
};

template <class D>
class SplitInterleavedDataInterface : public ArrayDataInterface<D, ComplexArray<D> > {
 public:
  SplitInterleavedDataInterface(int n, bool planar = true) : ArrayDataInterface<D, ComplexArray<D> >(n) {
    this->in = new ComplexArray<D>(n, planar);
    this->out = new ComplexArray<D>(n, planar);
  }
};

template <class D>
class PlannarizedDataInterface : public ArrayDataInterface<D, PlannarizedComplexArray<5, D> > {
 public:
  explicit PlannarizedDataInterface(int n) : ArrayDataInterface<D, PlannarizedComplexArray<5, D> >(n) {
    this->in = new PlannarizedComplexArray<5, D>(n);
    this->out = new PlannarizedComplexArray<5, D>(n);
  }
};

#endif
