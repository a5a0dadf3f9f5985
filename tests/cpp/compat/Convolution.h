/* Interface-compatible subset of ESTL's Convolution.h (Convolution.h:15-28):
 * the Data2D<T> and Convolution2D<T> interfaces that Convolution2D_FFT and
 * Convolution2D_FFT_CUDA implement.  The reference header also includes every
 * backend through FFTs.h (OpenCL included), which cannot be compiled here. */
#ifndef CONVOLUTION_H
#define CONVOLUTION_H

template <class T>
class Data2D {
 public:
  virtual int getWidth() = 0;
  virtual int getHeight() = 0;
  virtual T getPixel(int x, int y) = 0;
  virtual void setPixel(int x, int y, T value) = 0;
  virtual ~Data2D() {}
};

template <class T>
class Convolution2D {
 public:
  virtual void convolve(bool correlate = false) = 0;
  virtual ~Convolution2D() {}
};

#endif  // CONVOLUTION_H
