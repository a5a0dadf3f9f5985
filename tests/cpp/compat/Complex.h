/* Interface-compatible stand-in for ESTL's Complex.h (test infrastructure).
 *
 * The GPU test box has no copy of the reference, so the C++ plugin driver is
 * built there against these declarations, which keep the names and meaning of
 * the reference's plugin-facing types (Complex<R>, ComplexArray<D>,
 * AlignedArray<D>; Complex.h:17-32,52-95,156-192) in code of this project.
 * In this container the same driver is also compiled against the reference's
 * own headers (tests/test_plugin_cpp.py).
 */
#ifndef CCOMPLEX_H_
#define CCOMPLEX_H_

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <string>

template <class D>
class AlignedArray {
 public:
  explicit AlignedArray(int n) : raw(new unsigned char[(size_t)n * sizeof(D) + 31]) {
    alignedData = (D*)(((size_t)raw + 31) & ~(size_t)31);
  }
  ~AlignedArray() { delete[] raw; }
  D& operator[](int i) { return alignedData[i]; }
  D* alignedData;

 private:
  unsigned char* raw;
};

template <class R>
class Complex {
 public:
  Complex() {}
  Complex(R re) : r(re), i((R)0) {}
  Complex(R re, R im) : r(re), i(im) {}
  R getReal() const { return r; }
  R getImaginary() const { return i; }
  Complex getConjugate() const { return Complex(r, -i); }
  R getNormSquared() const { return r * r + i * i; }
  std::string toString() const {
    char b[96];
    snprintf(b, sizeof b, "(%f, %f)", (double)r, (double)i);
    return b;
  }
  Complex operator+(const Complex& o) const { return Complex(r + o.r, i + o.i); }
  Complex operator-(const Complex& o) const { return Complex(r - o.r, i - o.i); }
  Complex operator*(const Complex& o) const { return Complex(r * o.r - i * o.i, r * o.i + i * o.r); }

 private:
  R r, i;
};

/* Block-planar complex array: element i's real part at float
 * ((i >> 5) << 6) | (i & 31), its imaginary part 32 floats later
 * (interface of PlannarizedComplexArray<5, D>). */
template <int LEVEL, class D>
class PlannarizedComplexArray {
 public:
  explicit PlannarizedComplexArray(int n) : size(n), data(new AlignedArray<D>(2 * (((n + (1 << LEVEL) - 1) >> LEVEL) << LEVEL))) {}
  ~PlannarizedComplexArray() { delete data; }
  D* getData() { return &(*data)[0]; }
  int getSize() const { return size; }
  void setElement(int k, Complex<D> v) {
    (*data)[pos(k, 0)] = v.getReal();
    (*data)[pos(k, 1)] = v.getImaginary();
  }
  Complex<D> getElement(int k) { return Complex<D>((*data)[pos(k, 0)], (*data)[pos(k, 1)]); }

 private:
  static int pos(int k, int e) { return ((k >> LEVEL) << (LEVEL + 1)) | (e << LEVEL) | (k & ((1 << LEVEL) - 1)); }
  int size;
  AlignedArray<D>* data;
};

/* Interleaved (planar = false) or fully planar complex array. */
template <class D>
class ComplexArray {
 public:
  ComplexArray(int n, bool planar = true) : data(new AlignedArray<D>(2 * n)), size(n), planar(planar) {}
  ~ComplexArray() { delete data; }
  D* getData() { return &(*data)[0]; }
  void setElement(int k, Complex<D> v) {
    if (planar) {
      (*data)[k] = v.getReal();
      (*data)[size + k] = v.getImaginary();
    } else {
      (*data)[2 * k] = v.getReal();
      (*data)[2 * k + 1] = v.getImaginary();
    }
  }
  Complex<D> getElement(int k) {
    return planar ? Complex<D>((*data)[k], (*data)[size + k]) : Complex<D>((*data)[2 * k], (*data)[2 * k + 1]);
  }
  int getSize() const { return size; }

 private:
  AlignedArray<D>* data;
  int size;
  bool planar;
};

#endif
